// rsg_tick.cuh -- device implementation of one RocketSim Arena::Step tick.
//
// One warp advances one arena; the warps of a block step through the parts of a
// tick together, and work that is independent within an arena (wheels, cars,
// bodies, pads, narrow-phase candidates) is spread over lanes and warps.  The
// per-arena algorithm restates RocketSim v2.2's
// tick (src/Sim/Arena/Arena.cpp:689-756) including the parts of Bullet 3.24
// that decide its results: the voxel broadphase pair order, manifold creation
// order, the island quicksort that orders solver rows, 4-point manifolds, the
// sequential-impulse solver with split impulse and RocketSim's averaged
// ball-world contact.  Citations are <file>:<line> in the RocketSim tree; B/ is
// libsrc/bullet3-3.24/.
#pragma once
#include <cstdint>

#include "../../include/rocketsim_gb300.h"
#include "rsg_consts.cuh"
#include "rsg_layout.h"
#include "rsg_math.cuh"
#include "rsg_mesh.h"

namespace rsg {

#if !defined(__CUDACC__)
#error "rsg_tick.cuh is device code"
#endif
#define RSG_D __device__ __forceinline__
#define RSG_DN static __device__ __noinline__

__constant__ Curve c_curves[CV_COUNT] = RSG_CURVES_INIT;

// Optional per-phase cycle counters of lane 0 (compiled in only with -DRSG_PHASE_TIMERS).
#if defined(RSG_PHASE_TIMERS)
__device__ unsigned long long g_phase_cycles[64];
#define RSG_PHASE_BEGIN long long rsg_t_last_ = clock64()
#define RSG_PHASE(i)                                                                   \
    do {                                                                               \
        if (lane == 0) {                                                               \
            long long t_ = clock64();                                                  \
            atomicAdd(&g_phase_cycles[i], (unsigned long long)(t_ - rsg_t_last_));     \
            rsg_t_last_ = t_;                                                          \
        }                                                                              \
    } while (0)
// Sub-steps of lane-0-only code.
#define RSG_L0_BEGIN long long rsg_l_last_ = clock64()
#define RSG_L0(i)                                                                                   \
    do {                                                                                            \
        long long t_ = clock64();                                                                   \
        atomicAdd(&g_phase_cycles[i], (unsigned long long)(t_ - rsg_l_last_));                      \
        rsg_l_last_ = t_;                                                                           \
    } while (0)
// Block-level sub-steps, timed on thread 0 after each barrier, weighted by the block's arenas.
#define RSG_SUB_BEGIN long long rsg_s_last_ = clock64()
#define RSG_SUB(i)                                                                                  \
    do {                                                                                            \
        if (tid == 0) {                                                                             \
            long long t_ = clock64();                                                               \
            atomicAdd(&g_phase_cycles[i], (unsigned long long)((t_ - rsg_s_last_) * B.nact));       \
            rsg_s_last_ = t_;                                                                       \
        }                                                                                           \
    } while (0)
#else
#define RSG_PHASE_BEGIN
#define RSG_PHASE(i)
#define RSG_SUB_BEGIN
#define RSG_SUB(i)
#define RSG_L0_BEGIN
#define RSG_L0(i)
#endif
__constant__ float c_respawn_locs[4][2] = {{-2304, -4608}, {-2688, -4608}, {2304, -4608}, {2688, -4608}};

struct DevMesh {
    const float* tv;  // 9 floats per triangle
    const QNode* nodes;
    const Subtree* sub;
    const TriInfo* info;
    const uint8_t* cells;
    const QNode* lg_block;  // leaf grid (see HostMesh): 64-byte cell blocks
    const QNode* lg_over;
    const QNode* sub_grp;  // box of each run of 32 subtree headers
    int nsub_grp;
    int lg_shift[3], lg_n[3];
    int ntri, nnodes, nsub;
    V3 bvh_min, bvh_max, quant, aabb_min, aabb_max;
};
static_assert(sizeof(QNode) == 16, "leaf grid records are read as uint4");
static_assert(sizeof(Subtree) == 20, "subtree headers are read as five words");
struct DevGrid {
    V3 mn;
    float cell;
    int nx, ny, nz;
};

struct DevEvent {
    uint32_t kind;
    uint32_t tick_lo, tick_hi;
    uint32_t a, b, flag;
};

// Everything a kernel needs to reach one batch (passed by value)
struct BatchView {
    int A, MC;  // arenas, car slots per arena
    int has_arena;
    float dt;
    MutatorsDev mut;
    const float4* pad_cfg;  // per pad: position (uu) and is_big (ArenaConfig's pads or the soccar ones)
    int npads, custom_pads;  // pad count; custom pads skip BoostPadGrid (Arena.cpp:724-731)
    int no_ball_rot;         // ArenaConfig::noBallRot
    int heatseeker;          // GameMode::HEATSEEKER
    int lanes_per_car;       // threads per car in the vehicle update after the rays (1, 2 or 4)
    uint32_t* rec;  // A records of rec_words(MC) words
    int rec_words;
    uint32_t* au;   // [AU_COUNT][A]
    const CarCfgDev* cfgs;
    DevEvent* events;
    uint32_t event_mask;
    DevMesh mesh;
    DevGrid grid;
    unsigned char* tick_scratch;  // per warp slot: the working-set parts the tick kernel keeps out of shared memory
    int scratch_slots;            // warp slots in tick_scratch
};

constexpr int OBJ_MESH = 0, OBJ_PLANE0 = 1, OBJ_BALL = 5, OBJ_CAR0 = 6;
enum ActState { ACTIVE_TAG = 1, ISLAND_SLEEPING = 2, WANTS_DEACTIVATION = 3, DISABLE_DEACTIVATION = 4, DISABLE_SIMULATION = 5 };

// Per-arena capacities of the world-step scratch for `mc` car slots: every
// dynamic object can pair with the mesh and the 4 planes and with every other
// dynamic object; a manifold holds at most 4 points.
constexpr int MAX_DYN = MAX_CARS + 1;
constexpr int MAX_PAIRS = 5 * MAX_DYN + MAX_DYN * (MAX_CARS) / 2;
struct ArenaCaps {
    int pairs, points, rows;
};
RSG_HD ArenaCaps arena_caps(int mc) {
    int nd = mc + 1;
    ArenaCaps c;
    c.pairs = 5 * nd + nd * (nd - 1) / 2;
    c.points = 12 * nd;
    c.rows = c.points + nd;
    return c;
}

struct Body {
    Xf xf, interp;
    V3 lin_vel, ang_vel, total_force, total_torque;
    float inv_mass;
    V3 inv_inertia_local;
    M3 inv_inertia_world;
    float lin_damping;
    int act;
    bool no_rot, no_contact_response;
    float friction, restitution;
    V3 bp_min, bp_max;
    int ci, cj, ck;
    uint32_t cell, cell_seq;
    int n_special;
    float sp_friction, sp_restitution, sp_total_dist;
    V3 sp_total_normal;

    RSG_D void update_inertia() { inv_inertia_world = scaled(xf.b, inv_inertia_local) * transpose(xf.b); }
    RSG_D bool is_active() const { return act != ISLAND_SLEEPING && act != DISABLE_SIMULATION; }
    RSG_D V3 vel_at(V3 rel) const { return lin_vel + cross(ang_vel, rel); }
    RSG_D void apply_central_impulse(V3 imp) { lin_vel += imp * inv_mass; }
    RSG_D void apply_impulse(V3 imp, V3 rel) {
        if (inv_mass != 0.f) {
            apply_central_impulse(imp);
            ang_vel += inv_inertia_world * cross(rel, imp);
        }
    }
    RSG_D float impulse_denom(V3 pos, V3 n) const {
        V3 r0 = pos - xf.o;
        V3 c0 = cross(r0, n);
        V3 vec = cross(c0 * inv_inertia_world, r0);
        return inv_mass + dot(n, vec);
    }
};

struct WheelRT {
    V3 contact_normal, contact_point, hard_point, dir_ws, axle_ws, vel_at_contact, impulse;
    M3 wbasis;
    float susp_len, susp_rel_vel, clipped_inv_dot, susp_force;
    int ground;
    bool in_contact, contact_world;
};

struct Car {
    Body rb;
    const CarCfgDev* cfg;
    uint32_t flags, id, cc_other;
    int obj;
    float steer, pushback[4], latf[4], longf[4], engine, brake;
    V3 flip_rel;
    float jump_time, flip_time, air_time, air_time_sj, boost, time_since_boost, boosting_time, supersonic_time;
    float handbrake, autoflip_timer, autoflip_scale, cc_cooldown, demo_timer;
    V3 wc_normal, bhi_rel, bhi_ballpos, bhi_extra;
    uint64_t bhi_hit, bhi_extra_tick, ticks_since;
    float ctrl[5], last_ctrl[5];
    M3 rot;  // CarState::rotMat as basis rows
    V3 vel_cache;
    WheelRT w[4];

    RSG_D bool f(uint32_t m) const { return (flags & m) != 0; }
    RSG_D void setf(uint32_t m, bool v) { flags = v ? (flags | m) : (flags & ~m); }
    RSG_D V3 fwd() const { return rot.col(0); }
    RSG_D V3 right() const { return rot.col(1); }
    RSG_D V3 up() const { return rot.col(2); }
};

struct Pad {
    bool active;
    float cooldown;
    int cur_locked;
    uint32_t prev_locked;
};

struct MPoint {
    V3 local_a, local_b, pos_a, pos_b, normal;
    float dist, friction, restitution;
    bool special;
};
struct Manifold {
    int8_t body0, body1, n, island;
    float breaking;
    int8_t pt[4];
};

struct Row;
struct SBody;

// One arena's working state during a launch.  It lives in shared memory (one
// region per warp); the arrays are carved out of the same region, or (the parts
// the tick kernel's layout keeps out of shared memory) out of the warp's global
// scratch, with sizes from arena_caps(MC).
struct Ctx {
    DevEvent* ev;         // this arena's event slots
    uint32_t event_mask;  // bit k set: record events of kind k
    uint64_t ball_ticks;
    int ncars;
    int order[MAX_CARS];
    Car* cars;
    Body ball;
    V3 ball_cache;
    float hs_dir, hs_speed, hs_time;  // BallState::hsInfo (heatseeker)
    Pad* pads;
    uint64_t tick;
    uint32_t seq;
    bool stepped;
    uint32_t err;
    int nevents;
    float solver_dt;
    float ball_r, ball_breaking;  // ball radius (Bullet units) and its contact breaking threshold
    int serial;  // the pre-tick of this tick runs car by car in update order
    const Subtree* sub;  // BVH subtree headers (the block's shared-memory copy when there is one)
    int on_car;  // a wheel rests on another car: the car logic after the rays runs in update order
    // scratch of one world step
    int npairs, cap_pairs;
    int8_t* pair0;
    int8_t* pair1;
    int nman, npts, cap_pts;
    struct Manifold* man;
    MPoint* pts;
    SBody* sb;
    Row* rows_c;
    Row* rows_f;
    int cap_rows;
    // narrow-phase work lists: pair kinds, flattened candidate offsets, mesh candidates per
    // dynamic object, and the results of one round of candidate tests
    int8_t* pkind;
    int16_t* flat_off;
    int16_t* flat_n;
    int* cand_tri;
    int16_t* cand_n;
    struct CandRes* cand_res;
    uint16_t* qbox;    // [MAX_DYN][6] quantized query box of each mesh pair (min, max)
    int16_t* hdr_list; // [MAX_DYN][HDR_LIST] overlapping subtree headers in header order
    int16_t* hdr_n;    // [MAX_DYN], -1 when the list overflowed
    int nflat;
    uint32_t warn;
    // the solver batch planned on lane 0 and set up on the warp: solver bodies (object ids in island
    // order), (manifold, point) of every contact row in row order, bodies with special contacts
    int solve_nb, solve_nc, solve_nsp;
    int* solve_bodies;
    int* solve_plan;
    int16_t* solve_perm;  // rows by solver-body component: contact rows, friction rows, their two start lists
    int solve_ncomp;
    int8_t sb_of[MAX_CARS + 1];
    int8_t solve_special[MAX_CARS + 1];

    RSG_D Body& body(int o) { return o == OBJ_BALL ? ball : cars[o - OBJ_CAR0].rb; }
};

RSG_D bool is_static_obj(int o) { return o < OBJ_BALL; }

// ---------------------------------------------------------------- geometry consts
struct PlaneC {
    V3 n, origin, raw_min, raw_max, bp_min, bp_max;
};
RSG_D void plane_const(int p, PlaneC& out) {
    const float H = RL::ARENA_HEIGHT, EX = RL::ARENA_EXTENT_X;
    V3 pos, nrm;
    if (p == 0) { pos = V3(0, 0, 0); nrm = V3(0, 0, 1); }
    else if (p == 1) { pos = V3(0, 0, H); nrm = V3(0, 0, -1); }
    else if (p == 2) { pos = V3(-EX, 0, H / 2); nrm = V3(1, 0, 0); }
    else { pos = V3(EX, 0, H / 2); nrm = V3(-1, 0, 0); }
    out.n = normalized(nrm);
    out.origin = pos * RL::UU_TO_BT;
    V3 mn(-BT_LARGE, -BT_LARGE, -BT_LARGE), mx(BT_LARGE, BT_LARGE, BT_LARGE);
    int ax = fabsf(out.n.x) > 0.5f ? 0 : (fabsf(out.n.y) > 0.5f ? 1 : 2);
    bool back = out.n[ax] < 0;
    mn[ax] = out.origin[ax] + (0.f - 0.2f);
    mx[ax] = out.origin[ax] + (0.f + 0.2f);
    if (back) mx[ax] = BT_LARGE; else mn[ax] = -BT_LARGE;
    out.raw_min = mn;
    out.raw_max = mx;
    out.bp_min = mn - V3(0.02f, 0.02f, 0.02f);
    out.bp_max = mx + V3(0.02f, 0.02f, 0.02f);
}

// ---------------------------------------------------------------- mesh queries
RSG_D void tri_load(const DevMesh& m, int t, V3 v[3]) {
    const float* p = m.tv + (size_t)t * 9;
#if defined(__CUDA_ARCH__)
    v[0] = V3(__ldg(p + 0), __ldg(p + 1), __ldg(p + 2));
    v[1] = V3(__ldg(p + 3), __ldg(p + 4), __ldg(p + 5));
    v[2] = V3(__ldg(p + 6), __ldg(p + 7), __ldg(p + 8));
#else
    v[0] = V3(p[0], p[1], p[2]);
    v[1] = V3(p[3], p[4], p[5]);
    v[2] = V3(p[6], p[7], p[8]);
#endif
}
RSG_D void node_load(const DevMesh& m, int i, uint16_t qmin[3], uint16_t qmax[3], int& esc) {
#if defined(__CUDA_ARCH__)
    const uint4 raw = __ldg(reinterpret_cast<const uint4*>(m.nodes) + i);
    qmin[0] = raw.x & 0xffff; qmin[1] = raw.x >> 16; qmin[2] = raw.y & 0xffff;
    qmax[0] = raw.y >> 16; qmax[1] = raw.z & 0xffff; qmax[2] = raw.z >> 16;
    esc = (int)raw.w;
#else
    const QNode& n = m.nodes[i];
    for (int k = 0; k < 3; k++) { qmin[k] = n.qmin[k]; qmax[k] = n.qmax[k]; }
    esc = n.esc_or_tri;
#endif
}
RSG_D void node_load_ptr(const QNode* base, int i, uint16_t qmin[3], uint16_t qmax[3], int& w) {
    const uint4 raw = __ldg(reinterpret_cast<const uint4*>(base) + i);
    qmin[0] = raw.x & 0xffff; qmin[1] = raw.x >> 16; qmin[2] = raw.y & 0xffff;
    qmax[0] = raw.y >> 16; qmax[1] = raw.z & 0xffff; qmax[2] = raw.z >> 16;
    w = (int)raw.w;
}
RSG_D void quantize(const DevMesh& m, uint16_t* out, V3 p, bool is_max) {
    V3 v = (p - m.bvh_min) * m.quant;
    if (is_max) {
        out[0] = (uint16_t)(((uint16_t)(v.x + 1.f)) | 1);
        out[1] = (uint16_t)(((uint16_t)(v.y + 1.f)) | 1);
        out[2] = (uint16_t)(((uint16_t)(v.z + 1.f)) | 1);
    } else {
        out[0] = (uint16_t)(((uint16_t)(v.x)) & 0xfffe);
        out[1] = (uint16_t)(((uint16_t)(v.y)) & 0xfffe);
        out[2] = (uint16_t)(((uint16_t)(v.z)) & 0xfffe);
    }
}
RSG_D void quantize_clamp(const DevMesh& m, uint16_t* out, V3 p, bool is_max) {
    quantize(m, out, vmin(vmax(p, m.bvh_min), m.bvh_max), is_max);
}
RSG_D V3 unquantize(const DevMesh& m, const uint16_t* q) {
    V3 o((float)q[0] / m.quant.x, (float)q[1] / m.quant.y, (float)q[2] / m.quant.z);
    return o + m.bvh_min;
}
RSG_D bool qov(const uint16_t* a0, const uint16_t* a1, const uint16_t* b0, const uint16_t* b1) {
    bool o = true;
    o = (a0[0] > b1[0] || a1[0] < b0[0]) ? false : o;
    o = (a0[2] > b1[2] || a1[2] < b0[2]) ? false : o;
    o = (a0[1] > b1[1] || a1[1] < b0[1]) ? false : o;
    return o;
}

// walkStacklessQuantizedTreeCacheFriendly (btQuantizedBvh.cpp:551-575): subtree headers in order,
// the nodes of each overlapping subtree in order.
RSG_D void subtree_load(const DevMesh& m, int s, uint16_t qmin[3], uint16_t qmax[3], int& root, int& size) {
    const Subtree* st = m.sub + s;
    for (int k = 0; k < 3; k++) {
        qmin[k] = __ldg(&st->qmin[k]);
        qmax[k] = __ldg(&st->qmax[k]);
    }
    root = __ldg(&st->root);
    size = __ldg(&st->size);
}
RSG_D void subtree_load_at(const Subtree* st, uint16_t qmin[3], uint16_t qmax[3], int& root, int& size) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(st);
    uint32_t w0 = w[0], w1 = w[1], w2 = w[2];
    qmin[0] = w0 & 0xffff; qmin[1] = w0 >> 16; qmin[2] = w1 & 0xffff;
    qmax[0] = w1 >> 16; qmax[1] = w2 & 0xffff; qmax[2] = w2 >> 16;
    root = (int)w[3];
    size = (int)w[4];
}
template <class F>
RSG_D void subtree_walk(const DevMesh& m, const uint16_t* qa, const uint16_t* qb, int root, int size, F&& f) {
    int cur = root, end = root + size;
    while (cur < end) {
        uint16_t nmin[3], nmax[3];
        int esc;
        node_load(m, cur, nmin, nmax, esc);
        bool ov = qov(qa, qb, nmin, nmax);
        bool leaf = esc >= 0;
        if (leaf && ov) f(esc);
        if (ov || leaf) cur++;
        else cur += -esc;
    }
}
template <class F>
RSG_D void mesh_query_aabb(const DevMesh& m, V3 mn, V3 mx, F&& f) {
    uint16_t qa[3], qb[3];
    quantize_clamp(m, qa, mn, false);
    quantize_clamp(m, qb, mx, true);
    for (int s = 0; s < m.nsub; s++) {
        uint16_t smin[3], smax[3];
        int root, size;
        subtree_load(m, s, smin, smax, root, size);
        if (!qov(qa, qb, smin, smax)) continue;
        subtree_walk(m, qa, qb, root, size, f);
    }
}

// walkStacklessQuantizedTreeAgainstRay (btQuantizedBvh.cpp:436-548).  A node is entered when its
// quantized box overlaps the ray's and the ray meets its unquantized box (btRayAabb2); the
// triangles reported are the leaves that pass both tests, in node order.  The leaf grid gives that
// same set without the walk: a leaf that passes overlaps the ray's quantized box, so it is listed
// in one of the cells that box touches (it is taken from the first such cell only), and its
// ancestors pass whenever it does (their boxes contain its box).  The accepted leaves are sorted
// back into node order; more than RAY_GRID_MAX of them falls back to the walk.
struct RaySlab {
    V3 src, inv;
    float lambda_max;
    unsigned sg0, sg1, sg2;
    uint16_t qa[3], qb[3];
};
RSG_D void ray_slab_setup(const DevMesh& m, V3 src, V3 dst, RaySlab& r) {
    V3 dir = safe_normalized(dst - src);
    r.src = src;
    r.lambda_max = dot(dir, dst - src);
    r.inv = V3(dir.x == 0.f ? BT_LARGE : 1.f / dir.x, dir.y == 0.f ? BT_LARGE : 1.f / dir.y,
               dir.z == 0.f ? BT_LARGE : 1.f / dir.z);
    r.sg0 = r.inv.x < 0.f;
    r.sg1 = r.inv.y < 0.f;
    r.sg2 = r.inv.z < 0.f;
    quantize_clamp(m, r.qa, vmin(src, dst), false);
    quantize_clamp(m, r.qb, vmax(src, dst), true);
}
RSG_D bool ray_node_test(const DevMesh& m, const RaySlab& r, const uint16_t* nmin, const uint16_t* nmax) {
    if (!qov(r.qa, r.qb, nmin, nmax)) return false;
    V3 b0 = unquantize(m, nmin), b1 = unquantize(m, nmax);
    const V3 src = r.src, inv = r.inv;
    float tmin = ((r.sg0 ? b1 : b0).x - src.x) * inv.x;
    float tmax = ((r.sg0 ? b0 : b1).x - src.x) * inv.x;
    float tymin = ((r.sg1 ? b1 : b0).y - src.y) * inv.y;
    float tymax = ((r.sg1 ? b0 : b1).y - src.y) * inv.y;
    if ((tmin > tymax) || (tymin > tmax)) return false;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = ((r.sg2 ? b1 : b0).z - src.z) * inv.z;
    float tzmax = ((r.sg2 ? b0 : b1).z - src.z) * inv.z;
    if ((tmin > tzmax) || (tzmin > tmax)) return false;
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    return (tmin < r.lambda_max) && (tmax > 0.f);
}
constexpr int RAY_GRID_MAX = 6;
// The triangles a ray reports, from the leaf grid, in node order: their count (keys in key[]:
// (rank << 16) | triangle, sorted by rank), or -1 when there are more than RAY_GRID_MAX (the caller
// then walks the tree).  key[] is indexed statically so it stays in registers.
RSG_D int ray_grid_tris(const DevMesh& m, const RaySlab& r, int (&key)[RAY_GRID_MAX]) {
    int c0[3], c1[3];
    for (int k = 0; k < 3; k++) {
        c0[k] = r.qa[k] >> m.lg_shift[k];
        c1[k] = r.qb[k] >> m.lg_shift[k];
    }
    int n = 0;
    const uint4* blocks = reinterpret_cast<const uint4*>(m.lg_block);
    const uint4* over = reinterpret_cast<const uint4*>(m.lg_over);
    for (int x = c0[0]; x <= c1[0]; x++)
        for (int y = c0[1]; y <= c1[1]; y++)
            for (int z = c0[2]; z <= c1[2]; z++) {
                const uint32_t cell = ((uint32_t)x * m.lg_n[1] + y) * m.lg_n[2] + z;
                const uint4 hdr = __ldg(blocks + (size_t)cell * 4);
                const uint32_t count = hdr.x, off = hdr.y;
                for (uint32_t e = 0; e < count; e++) {  // one compact loop: the block's line stays in L1
                    const uint4 rec = e < 3 ? __ldg(blocks + (size_t)cell * 4 + 1 + e) : __ldg(over + off + (e - 3));
                    uint16_t nmin[3], nmax[3];
                    nmin[0] = rec.x & 0xffff; nmin[1] = rec.x >> 16; nmin[2] = rec.y & 0xffff;
                    nmax[0] = rec.y >> 16; nmax[1] = rec.z & 0xffff; nmax[2] = rec.z >> 16;
                    // the leaf's first cell inside the ray's cell range
                    int fx = nmin[0] >> m.lg_shift[0], fy = nmin[1] >> m.lg_shift[1], fz = nmin[2] >> m.lg_shift[2];
                    if ((fx > c0[0] ? fx : c0[0]) != x || (fy > c0[1] ? fy : c0[1]) != y ||
                        (fz > c0[2] ? fz : c0[2]) != z)
                        continue;
                    if (!ray_node_test(m, r, nmin, nmax)) continue;
                    if (n == RAY_GRID_MAX) return -1;
                    // insertion by rank (node order) with static indices: shift the larger keys up
                    int v = (int)rec.w;
#pragma unroll
                    for (int q = 0; q < RAY_GRID_MAX; q++) {
                        if (q < n && key[q] > v) { int t = key[q]; key[q] = v; v = t; }
                    }
#pragma unroll
                    for (int q = 0; q < RAY_GRID_MAX; q++)
                        if (q == n) key[q] = v;
                    n++;
                }
            }
    return n;
}
template <class F>
RSG_D void mesh_query_ray(const DevMesh& m, V3 src, V3 dst, F&& f) {
#if defined(RSG_PHASE_TIMERS)
    long long qt_ = clock64();
#define RSG_QT(i) do { long long t_ = clock64(); atomicAdd(&g_phase_cycles[i], (unsigned long long)(t_ - qt_)); qt_ = t_; } while (0)
#else
#define RSG_QT(i)
#endif
    RaySlab r;
    ray_slab_setup(m, src, dst, r);
    RSG_QT(35);
    if (m.lg_block) {
        int key[RAY_GRID_MAX];
        const int n = ray_grid_tris(m, r, key);
        RSG_QT(36);
        if (n >= 0) {
#pragma unroll
            for (int i = 0; i < RAY_GRID_MAX; i++)
                if (i < n) f(key[i] & 0xffff);
            RSG_QT(37);
#if defined(RSG_PHASE_TIMERS)
            atomicAdd(&g_phase_cycles[38], (unsigned long long)n);
#endif
            return;
        }
#if defined(RSG_PHASE_TIMERS)
        atomicAdd(&g_phase_cycles[39], 1ull);
#endif
    }
    int cur = 0;
    while (cur < m.nnodes) {
        uint16_t nmin[3], nmax[3];
        int esc;
        node_load(m, cur, nmin, nmax, esc);
        bool leaf = esc >= 0;
        bool rayov = ray_node_test(m, r, nmin, nmax);
        if (leaf && rayov) f(esc);
        if (rayov || leaf) cur++;
        else cur += -esc;
    }
}

// ---------------------------------------------------------------- ray tests
// btTriangleRaycastCallback::processTriangle (B/.../NarrowPhaseCollision/btRaycastCallback.cpp:35-118)
RSG_D bool ray_triangle(V3 from, V3 to, const V3 tv[3], float& hit_frac, V3& out_n) {
    V3 v10 = tv[1] - tv[0], v20 = tv[2] - tv[0];
    V3 n = cross(v10, v20);
    float dist = dot(tv[0], n);
    float da = dot(n, from) - dist;
    float db = dot(n, to) - dist;
    if (da * db >= 0.f) return false;
    float distance = da / (da - db);
    if (!(distance < hit_frac)) return false;
    float tol = len2(n) * -0.0001f;
    V3 point = lerp(from, to, distance);
    V3 v0p = tv[0] - point, v1p = tv[1] - point;
    if (!(dot(cross(v0p, v1p), n) >= tol)) return false;
    V3 v2p = tv[2] - point;
    if (!(dot(cross(v1p, v2p), n) >= tol)) return false;
    if (!(dot(cross(v2p, v0p), n) >= tol)) return false;
    n = normalized(n);
    out_n = (da <= 0.f) ? -n : n;
    hit_frac = distance;
    return true;
}
// btStaticPlaneShape::processAllTriangles (btStaticPlaneShape.cpp:56-87) fed to the ray callback
RSG_D bool ray_plane(const PlaneC& p, V3 from_w, V3 to_w, float& hit_frac, V3& out_n) {
    // the plane body has an identity basis, so world-to-object is a translation
    V3 from = from_w - p.origin, to = to_w - p.origin;
    V3 amin = vmin(from, to), amax = vmax(from, to);
    V3 he = (amax - amin) * 0.5f;
    float radius = len(he);
    V3 center = (amax + amin) * 0.5f;
    V3 t0, t1;
    plane_space(p.n, t0, t1);
    V3 pc = center - (dot(p.n, center) - 0.f) * p.n;
    bool any = false;
    V3 tri[3], n;
    tri[0] = pc + t0 * radius + t1 * radius;
    tri[1] = pc + t0 * radius - t1 * radius;
    tri[2] = pc - t0 * radius - t1 * radius;
    if (ray_triangle(from, to, tri, hit_frac, n)) { any = true; out_n = n; }
    tri[0] = pc - t0 * radius - t1 * radius;
    tri[1] = pc - t0 * radius + t1 * radius;
    tri[2] = pc + t0 * radius + t1 * radius;
    if (ray_triangle(from, to, tri, hit_frac, n)) { any = true; out_n = n; }
    return any;
}
// Rays against the ball / another car's box the way btCollisionWorld::rayTestSingleInternal casts
// them (btCollisionWorld.cpp:267-310): btSubsimplexConvexCast of a point against the car's box child
// (the car's compound keeps no child tree, Car.cpp:198) or the ball's sphere.  Defined after the
// simplex solver they share with GJK.
RSG_DN bool ray_cast_box(V3 from, V3 to, const Xf& box_xf, V3 he_margin, float& hit_frac, V3& out_n);
RSG_DN bool ray_cast_sphere(V3 from, V3 to, const Xf& xf, float radius, float& hit_frac, V3& out_n);


// ---------------------------------------------------------------- broadphase helpers
RSG_D void grid_idx(const DevGrid& g, V3 p, int& i, int& j, int& k) {
    V3 f = (p - g.mn) / g.cell;
    i = (int)f.x; j = (int)f.y; k = (int)f.z;
    i = i < 0 ? 0 : (i > g.nx - 1 ? g.nx - 1 : i);
    j = j < 0 ? 0 : (j > g.ny - 1 ? g.ny - 1 : j);
    k = k < 0 ? 0 : (k > g.nz - 1 ? g.nz - 1 : k);
}
RSG_D bool dyn_registered(const Body& b, int ci, int cj, int ck) {
    if (b.cell == 0xffffffffu) return false;
    int di = b.ci - ci, dj = b.cj - cj, dk = b.ck - ck;
    return di >= -1 && di <= 1 && dj >= -1 && dj <= 1 && dk >= -1 && dk <= 1;
}
// dynamic proxies registered in cell (ci,cj,ck) ordered like the cell's handle list
RSG_D int cell_dyn_list(Ctx& a, int ci, int cj, int ck, int* out) {
    int n = 0;
    if (dyn_registered(a.ball, ci, cj, ck)) out[n++] = OBJ_BALL;
    for (int i = 0; i < a.ncars; i++)
        if (dyn_registered(a.cars[i].rb, ci, cj, ck)) out[n++] = OBJ_CAR0 + i;
    for (int i = 1; i < n; i++) {  // insertion sort by cell-change sequence (stable)
        int v = out[i];
        uint32_t sv = a.body(v).cell_seq;
        int j = i - 1;
        while (j >= 0 && a.body(out[j]).cell_seq > sv) { out[j + 1] = out[j]; j--; }
        out[j + 1] = v;
    }
    return n;
}

// ---------------------------------------------------------------- vehicle
struct RayHit {
    bool hit;
    int obj;
    float frac;
    V3 normal, point;
};

RSG_D void car_child_xf(const Car& c, Xf& out) {
    Xf off = xf_identity();
    off.o = V3(c.cfg->off[0], c.cfg->off[1], c.cfg->off[2]);
    out = xf_mul(c.rb.xf, off);
}
RSG_D V3 car_he(const Car& c) { return V3(c.cfg->he[0], c.cfg->he[1], c.cfg->he[2]); }

RSG_DN RayHit cast_ray(const BatchView& bv, Ctx& a, V3 from, V3 to, int self_obj) {
#if defined(RSG_PHASE_TIMERS)
    long long ct_ = clock64();
#define RSG_CT(i) do { long long t_ = clock64(); atomicAdd(&g_phase_cycles[i], (unsigned long long)(t_ - ct_)); ct_ = t_; } while (0)
#else
#define RSG_CT(i)
#endif
    RayHit r;
    r.hit = false;
    float frac = 1.f;
    int obj = -1;
    V3 nrm;
    if (bv.has_arena) {
        mesh_query_ray(bv.mesh, from, to, [&](int t) {
            V3 tv[3];
            tri_load(bv.mesh, t, tv);
            V3 n;
            if (ray_triangle(from, to, tv, frac, n)) { obj = OBJ_MESH; nrm = n; }
        });
        RSG_CT(32);
        for (int p = 0; p < 4; p++) {
            // ray_plane's triangles lie in the plane and need the ray's ends on both sides of it
            // (da * db < 0 in ray_triangle); ends more than 0.01 on one side cannot hit
            const float H = RL::ARENA_HEIGHT * RL::UU_TO_BT, EX = RL::ARENA_EXTENT_X * RL::UU_TO_BT;
            float sa, sb;
            if (p == 0) { sa = from.z; sb = to.z; }
            else if (p == 1) { sa = H - from.z; sb = H - to.z; }
            else if (p == 2) { sa = from.x + EX; sb = to.x + EX; }
            else { sa = EX - from.x; sb = EX - to.x; }
            if ((sa > 0.01f && sb > 0.01f) || (sa < -0.01f && sb < -0.01f)) continue;
            PlaneC pl;
            plane_const(p, pl);
            V3 n;
            if (ray_plane(pl, from, to, frac, n)) { obj = OBJ_PLANE0 + p; nrm = n; }
        }
    }
    RSG_CT(33);
    int ci, cj, ck;
    grid_idx(bv.grid, from, ci, cj, ck);
    int dyn[MAX_CARS + 1];
    int nd = cell_dyn_list(a, ci, cj, ck, dyn);
    for (int k = 0; k < nd; k++) {
        int o = dyn[k];
        if (o == self_obj) continue;
        if (frac == 0.f) break;
        V3 n;
        if (o == OBJ_BALL) {
            if (ray_cast_sphere(from, to, a.ball.xf, a.ball_r, frac, n)) { obj = o; nrm = n; }
        } else {
            Car& c = a.cars[o - OBJ_CAR0];
            Xf bx = c.rb.xf;
            bx.o = xf_apply(c.rb.xf, V3(c.cfg->off[0], c.cfg->off[1], c.cfg->off[2]));
            V3 he = car_he(c) + V3(c.cfg->margin, c.cfg->margin, c.cfg->margin);
            if (ray_cast_box(from, to, bx, he, frac, n)) { obj = o; nrm = n; }
        }
    }
    RSG_CT(34);
    if (obj < 0) return r;
    if (!is_static_obj(obj) && a.body(obj).no_contact_response) return r;
    r.hit = true;
    r.obj = obj;
    r.frac = frac;
    r.normal = normalized(nrm);
    r.point = lerp(from, to, frac);
    return r;
}

RSG_D V3 static_origin(int o) {
    if (o == OBJ_MESH) return V3(0, 0, 0);
    PlaneC p;
    plane_const(o - OBJ_PLANE0, p);
    return p.origin;
}

RSG_D void wheel_ws(Car& c, int i) {  // btVehicleRL::updateWheelTransformsWS (btVehicleRL.cpp:110-118)
    WheelRT& w = c.w[i];
    w.in_contact = false;
    w.contact_world = false;
    w.hard_point = xf_apply(c.rb.xf, V3(c.cfg->conn[i][0], c.cfg->conn[i][1], c.cfg->conn[i][2]));
    w.dir_ws = c.rb.xf.b * V3(0, 0, -1);
    w.axle_ws = c.rb.xf.b * V3(0, -1, 0);
}
RSG_D void update_wheel_transform(Car& c, int i) {  // btVehicleRL::updateWheelTransform (btVehicleRL.cpp:66-94)
    wheel_ws(c, i);
    WheelRT& w = c.w[i];
    V3 up = -w.dir_ws;
    V3 right = w.axle_ws;
    V3 fwd = normalized(cross(up, right));
    float steer = i < 2 ? c.steer : 0.f;
    M3 sm = m_from_q(q_axis_angle(up, steer));
    M3 b2;
    for (int r = 0; r < 3; r++) {
        b2.r[r][1] = -right[r];
        b2.r[r][2] = up[r];
        b2.r[r][0] = fwd[r];
    }
    w.wbasis = sm * b2;
}

RSG_D float resolve_single_collision(Ctx& a, Body& b1, int obj2, V3 pos, V3 n, float distance) {
    V3 rel1 = pos - b1.xf.o;
    bool dyn2 = !is_static_obj(obj2);
    V3 o2 = dyn2 ? a.body(obj2).xf.o : static_origin(obj2);
    V3 rel2 = pos - o2;
    V3 v1 = b1.vel_at(rel1);
    V3 v2 = dyn2 ? a.body(obj2).vel_at(rel2) : V3(0, 0, 0);
    float rel_vel = dot(n, v1 - v2);
    float restitution = 0.f * -rel_vel;
    float pos_err = 0.2f * -distance / a.solver_dt;
    float vel_err = -(1.0f + restitution) * rel_vel;
    float d0 = b1.impulse_denom(pos, n);
    float d1 = dyn2 ? a.body(obj2).impulse_denom(pos, n) : 0.f;
    float jac = 1.f / (d0 + d1);
    float imp = pos_err * jac + vel_err * jac;
    return 0.f > imp ? 0.f : imp;
}

RSG_D void ray_cast_wheel(const BatchView& bv, Ctx& a, Car& c, int i) {  // btVehicleRL::rayCast (btVehicleRL.cpp:120-209)
    wheel_ws(c, i);
    WheelRT& w = c.w[i];
    int fb = i < 2 ? 0 : 1;
    float rest = c.cfg->rest[fb], radius = c.cfg->radius[fb];
    float travel_cm = (RL::MAX_SUSPENSION_TRAVEL * RL::UU_TO_BT) * 100;
    float travel = travel_cm / 100;
    float ray_len = rest + travel + radius - RL::SUSPENSION_SUBTRACTION;
    V3 src = w.hard_point;
    V3 dst = src + (w.dir_ws * ray_len);
    w.contact_point = dst;
    w.ground = -1;
    RayHit h = cast_ray(bv, a, src, dst, c.obj);
    if (h.hit) {
        w.contact_point = h.point;
        w.contact_normal = h.normal;
        w.in_contact = true;
        bool stat = is_static_obj(h.obj);
        w.contact_world = stat;
        w.ground = h.obj;
        V3 up = c.rb.xf.b.col(2);
        float trace = dot(w.hard_point - w.contact_point, up);
        w.susp_len = trace - radius;
        float lo = rest - travel, hi = rest + travel;
        w.susp_len = w.susp_len < lo ? lo : (hi < w.susp_len ? hi : w.susp_len);
        float denom = dot(w.contact_normal, up);
        V3 relpos = w.contact_point - c.rb.xf.o;
        w.vel_at_contact = c.rb.vel_at(relpos);
        float projv = dot(w.contact_normal, w.vel_at_contact);
        if (denom > 0.1f) {
            float inv = 1 / denom;
            w.susp_rel_vel = projv * inv;
            w.clipped_inv_dot = inv;
        } else {
            w.susp_rel_vel = 0;
            w.clipped_inv_dot = 10;
        }
        if (stat) {
            float thresh = (rest + radius) - RL::SUSPENSION_SUBTRACTION;
            if (trace < thresh) {
                float res = resolve_single_collision(a, c.rb, h.obj, h.point, h.normal, trace - thresh);
                c.pushback[i] = res / 4;
            }
        }
    } else {
        w.susp_len = rest + travel;
        w.susp_rel_vel = 0;
        w.contact_normal = -w.dir_ws;
        w.clipped_inv_dot = 1;
        c.pushback[i] = 0;
    }
}

RSG_D float resolve_single_bilateral(Ctx& a, Body& b1, V3 pos, int obj2, V3 normal) {  // btContactConstraint.cpp:103-150
    if (len2(normal) > 1.1f) return 0.f;
    bool dyn2 = !is_static_obj(obj2);
    V3 o2 = dyn2 ? a.body(obj2).xf.o : static_origin(obj2);
    V3 rel1 = pos - b1.xf.o;
    V3 rel2 = pos - o2;
    V3 v1 = b1.vel_at(rel1);
    V3 v2 = dyn2 ? a.body(obj2).vel_at(rel2) : V3(0, 0, 0);
    M3 w2a = transpose(b1.xf.b);
    M3 w2b = dyn2 ? transpose(a.body(obj2).xf.b) : M3();
    V3 aJ = w2a * cross(rel1, normal);
    V3 bJ = w2b * cross(rel2, -normal);
    V3 invIB = dyn2 ? a.body(obj2).inv_inertia_local : V3(0, 0, 0);
    float invMB = dyn2 ? a.body(obj2).inv_mass : 0.f;
    V3 m0 = b1.inv_inertia_local * aJ, m1 = invIB * bJ;
    float diag = b1.inv_mass + dot(m0, aJ) + invMB + dot(m1, bJ);
    float jinv = 1.f / diag;
    return -0.2f * dot(normal, v1 - v2) * jinv;
}

// btVehicleRL::calcFrictionImpulses (btVehicleRL.cpp:306-380) for wheel i (wheels are independent)
RSG_D void calc_friction_impulse(Ctx& a, Car& c, float dt, int i) {
    float fscale = (1.f / c.rb.inv_mass) / 3;
    {
        WheelRT& w = c.w[i];
        if (w.ground >= 0) {
            V3 axle = w.wbasis.col(1);
            V3 n = w.contact_normal;
            float proj = dot(axle, n);
            axle -= n * proj;
            axle = safe_normalized(axle);
            V3 fwd = safe_normalized(cross(n, axle));
            float side = resolve_single_bilateral(a, c.rb, w.contact_point, w.ground, axle);
            float roll;
            if (c.engine == 0) {
                if (c.brake) {
                    V3 crel = w.contact_point - c.rb.xf.o;
                    bool dyn2 = !is_static_obj(w.ground);
                    V3 v1 = c.rb.vel_at(crel);
                    V3 v2 = dyn2 ? a.body(w.ground).vel_at(crel) : V3(0, 0, 0);
                    float rv = dot(v1 - v2, fwd);
                    if (dt > (1 / 80.f)) {
                        float th = -(1 / (dt * 150.f)) + 0.8f;
                        if (fabsf(rv) < th) rv = 0;
                    }
                    const float MAGIC = 113.73963f;
                    float x = -rv * MAGIC;
                    float lo = -c.brake, hi = c.brake;
                    roll = x > lo ? x : lo;
                    roll = roll < hi ? roll : hi;
                } else {
                    roll = 0;
                }
            } else {
                roll = -c.engine / fscale;
            }
            V3 total = (fwd * roll * c.longf[i]) + (axle * side * c.latf[i]);
            w.impulse = total * fscale;
        } else {
            w.impulse = V3(0, 0, 0);
        }
    }
}

RSG_D V3 upwards_from_wheels(const Car& c) {  // btVehicleRL.cpp:397-410
    V3 sum(0, 0, 0);
    for (int i = 0; i < 4; i++)
        if (c.w[i].in_contact) sum += c.w[i].contact_normal;
    if (sum == V3(0, 0, 0)) return c.rb.xf.b.col(2);
    return safe_normalized(sum);
}

// btVehicleRL::updateSuspension (btVehicleRL.cpp:270-303): the force of wheel i
RSG_D void suspension_force(Car& c, int i) {
    {
        WheelRT& w = c.w[i];
        if (w.in_contact) {
            int fb = i < 2 ? 0 : 1;
            float force = (c.cfg->rest[fb] - w.susp_len) * RL::SUSPENSION_STIFFNESS * w.clipped_inv_dot;
            float damp = (w.susp_rel_vel < 0) ? RL::WHEELS_DAMPING_COMPRESSION : RL::WHEELS_DAMPING_RELAXATION;
            w.susp_force = force - (damp * w.susp_rel_vel);
            w.susp_force *= (i < 2) ? RL::SUSPENSION_FORCE_SCALE_FRONT : RL::SUSPENSION_FORCE_SCALE_BACK;
            if (w.susp_force < 0) w.susp_force = 0;
        } else {
            w.susp_force = 0;
        }
    }
}
// ... and the suspension impulses on the chassis, wheel by wheel in order
RSG_D void apply_suspension(Car& c, float dt) {
    for (int i = 0; i < 4; i++) {
        WheelRT& w = c.w[i];
        if (w.susp_force != 0) {
            V3 off = w.contact_point - c.rb.xf.o;
            float base = (w.susp_force * dt) + c.pushback[i];
            c.rb.apply_impulse(w.contact_normal * base, off);
        }
    }
}

RSG_D void apply_friction_impulses(Car& c, float dt) {  // btVehicleRL.cpp:383-395
    V3 up = c.rb.xf.b.col(2);
    for (int i = 0; i < 4; i++) {
        WheelRT& w = c.w[i];
        if (!is_zero(w.impulse)) {
            V3 off = w.contact_point - c.rb.xf.o;
            float d = dot(up, off);
            c.rb.apply_impulse(w.impulse * dt, off - up * d);
        }
    }
}

// The chassis velocity changes of wheel i's suspension impulse (apply_suspension) and friction
// impulse (apply_friction_impulses), each computed as Body::apply_impulse computes it.
struct ImpulseDeltas {
    V3 dvs, dws, dvf, dwf;
    bool son, fon;
};
RSG_D ImpulseDeltas wheel_impulse_deltas(const Car& c, int i, float dt) {
    ImpulseDeltas d;
    const WheelRT& w = c.w[i];
    const V3 off = w.contact_point - c.rb.xf.o;
    d.son = w.susp_force != 0;
    d.dvs = d.dws = d.dvf = d.dwf = V3(0, 0, 0);
    if (d.son) {
        const V3 imp = w.contact_normal * ((w.susp_force * dt) + c.pushback[i]);
        d.dvs = imp * c.rb.inv_mass;
        d.dws = c.rb.inv_inertia_world * cross(off, imp);
    }
    d.fon = !is_zero(w.impulse);
    if (d.fon) {
        const V3 up = c.rb.xf.b.col(2);
        const float dd = dot(up, off);
        const V3 imp = w.impulse * dt, rel = off - up * dd;
        d.dvf = imp * c.rb.inv_mass;
        d.dwf = c.rb.inv_inertia_world * cross(rel, imp);
    }
    return d;
}
RSG_D V3 shfl_v3(unsigned mask, V3 v, int src) {
    return V3(__shfl_sync(mask, v.x, src), __shfl_sync(mask, v.y, src), __shfl_sync(mask, v.z, src));
}

// ---------------------------------------------------------------- car logic (Car.cpp)
RSG_D float rs_maxf(float a, float b) { return (a > b) ? a : b; }
RSG_D float rs_minf(float a, float b) { return (a < b) ? a : b; }
RSG_D float rs_clampf(float v, float lo, float hi) { return rs_minf(rs_maxf(v, lo), hi); }
RSG_D int rs_sgn(float v) { return (v > 0) - (v < 0); }

// Car::_UpdateWheels (Car.cpp:339-484) in three parts: the car's handbrake, engine, brake and steer
// (computed by every thread of the car's group, stored by `store`), each wheel's friction curves,
// and the sticky force.
struct WheelsCommon {
    float absfs, real_throttle;
    bool world_contact;
};
RSG_D WheelsCommon update_wheels_car(Car& c, float dt, int nwc, float fwd_speed, float hb, bool store) {
    WheelsCommon wc;
    float absfs = fabsf(fwd_speed);
    bool world_contact = false;
    for (int i = 0; i < 4; i++) world_contact |= c.w[i].contact_world;
    if (c.f(F_CTRL_HB)) hb += RL::POWERSLIDE_RISE_RATE * dt;
    else hb -= RL::POWERSLIDE_FALL_RATE * dt;
    hb = rs_clampf(hb, 0, 1);
    float real_throttle = c.ctrl[0];
    float real_brake = 0;
    if (c.f(F_CTRL_BOOST) && c.boost > 0) real_throttle = 1;
    float engine, brake, steer;
    {
        float dss = curve_eval(c_curves[CV_DRIVE_TORQUE], absfs);
        float eng = real_throttle;
        if (!c.f(F_CTRL_HB)) {
            float at = fabsf(real_throttle);
            if (at >= RL::THROTTLE_DEADZONE) {
                if (absfs > RL::STOPPING_FORWARD_VEL && rs_sgn(real_throttle) != rs_sgn(fwd_speed)) {
                    real_brake = 1;
                    if (absfs > RL::BRAKING_NO_THROTTLE_SPEED_THRESH) eng = 0;
                }
            } else {
                eng = 0;
                real_brake = (absfs < RL::STOPPING_FORWARD_VEL) ? 1 : RL::COASTING_BRAKE_FACTOR;
            }
        }
        if (nwc < 3) dss /= 4;
        engine = eng * (RL::THROTTLE_TORQUE_AMOUNT * RL::UU_TO_BT) * dss;
        brake = real_brake * (RL::BRAKE_TORQUE_AMOUNT * RL::UU_TO_BT);
    }
    {
        bool tw = c.cfg->three_wheels != 0;
        steer = curve_eval(c_curves[tw ? CV_STEER_3W : CV_STEER], absfs);
        if (hb) steer += (curve_eval(c_curves[CV_POWERSLIDE_STEER], absfs) - steer) * hb;
        steer *= c.ctrl[1];
    }
    if (store) {
        c.handbrake = hb;
        c.engine = engine;
        c.brake = brake;
        c.steer = steer;
    }
    wc.absfs = absfs;
    wc.real_throttle = real_throttle;
    wc.world_contact = world_contact;
    return wc;
}
// reads the handbrake stored by update_wheels_car
RSG_D void update_wheel_friction(Car& c, const WheelsCommon& wc, int i) {
    WheelRT& w = c.w[i];
    if (w.ground >= 0) {
        V3 vel = c.rb.lin_vel, av = c.rb.ang_vel;
        V3 lat = w.wbasis.col(1);
        V3 lng = cross(lat, w.contact_normal);
        float in = 0;
        V3 wd = w.hard_point - c.rb.xf.o;
        V3 cv = (cross(av, wd) + vel) * RL::BT_TO_UU;
        float base = fabsf(dot(cv, lat));
        if (base > 5) in = base / (fabsf(dot(cv, lng)) + base);
        bool tw = c.cfg->three_wheels != 0;
        float latf = curve_eval(c_curves[tw ? CV_LAT_FRIC_3W : CV_LAT_FRIC], in);
        float longf = curve_eval(c_curves[CV_LONG_FRIC], in);
        if (c.handbrake) {
            float hb = c.handbrake;
            latf *= (curve_eval(c_curves[CV_HB_LAT], in) - 1) * hb + 1;
            longf *= (curve_eval(c_curves[CV_HB_LONG], in) - 1) * hb + 1;
        } else {
            longf = 1;
        }
        if (!(wc.real_throttle != 0)) {
            float ns = curve_eval(c_curves[CV_NON_STICKY], w.contact_normal.z);
            latf *= ns;
            longf *= ns;
        }
        c.latf[i] = latf;
        c.longf[i] = longf;
    }
}
RSG_D void update_wheels_sticky(Car& c, const WheelsCommon& wc) {
    if (wc.world_contact) {
        V3 updir = upwards_from_wheels(c);
        bool full = (wc.real_throttle != 0) || (wc.absfs > RL::STOPPING_FORWARD_VEL);
        float sfs = c.cfg->three_wheels ? 0 : 0.5f;
        if (full) sfs += 1 - fabsf(updir.z);
        c.rb.total_force += updir * sfs * (RL::GRAVITY_Z * RL::UU_TO_BT) * RL::CAR_MASS_BT;
    }
}

RSG_D void update_boost(Car& c, float dt, const MutatorsDev& m) {  // Car::_UpdateBoost (Car.cpp:486-533)
    bool has = c.boost > 0;
    bool boosting = c.f(F_BOOSTING);
    if (has) {
        if (boosting) boosting = (c.f(F_CTRL_BOOST) || c.boosting_time < RL::BOOST_MIN_TIME);
        else if (c.f(F_CTRL_BOOST)) boosting = true;
    } else {
        boosting = false;
    }
    c.setf(F_BOOSTING, boosting);
    if (boosting) c.boosting_time += dt;
    else c.boosting_time = 0;
    if (boosting) {
        c.boost = rs_maxf(c.boost - m.boost_used_per_second * dt, 0);
        c.rb.total_force += (c.f(F_ON_GROUND) ? m.boost_accel_ground : m.boost_accel_air) * RL::UU_TO_BT * c.fwd() *
                            RL::CAR_MASS_BT;
        c.time_since_boost = 0;
    } else {
        c.time_since_boost += dt;
        if (m.recharge_boost)
            if (c.time_since_boost >= m.recharge_delay) c.boost += m.recharge_per_second * dt;
    }
    c.boost = rs_minf(c.boost, RL::BOOST_MAX);
}

RSG_D void update_jump(Car& c, float dt, bool pressed, const MutatorsDev& m) {  // Car::_UpdateJump (Car.cpp:535-582)
    if (c.f(F_ON_GROUND) && !c.f(F_JUMPING)) {
        if (c.f(F_HAS_JUMPED) && c.jump_time < RL::JUMP_MIN_TIME + RL::JUMP_RESET_TIME_PAD) {
        } else {
            c.setf(F_HAS_JUMPED, false);
            c.jump_time = 0;
        }
    }
    if (c.f(F_JUMPING)) {
        c.setf(F_JUMPING, c.jump_time < RL::JUMP_MIN_TIME || (c.f(F_CTRL_JUMP) && c.jump_time < RL::JUMP_MAX_TIME));
    } else if (c.f(F_ON_GROUND) && pressed) {
        c.setf(F_JUMPING, true);
        c.jump_time = 0;
        c.rb.apply_central_impulse(c.up() * m.jump_immediate_force * RL::UU_TO_BT * RL::CAR_MASS_BT);
    }
    if (c.f(F_JUMPING)) {
        c.setf(F_HAS_JUMPED, true);
        V3 tf = c.up() * m.jump_accel;
        if (c.jump_time < RL::JUMP_MIN_TIME) tf *= 0.62f;
        c.rb.total_force += tf * RL::UU_TO_BT * RL::CAR_MASS_BT;
    }
    if (c.f(F_JUMPING) || c.f(F_HAS_JUMPED)) c.jump_time += dt;
}

RSG_D void update_air_torque(Car& c, bool update_air_control) {  // Car::_UpdateAirTorque (Car.cpp:584-669)
    V3 pitch_right = -c.right(), yaw_up = c.up(), roll_fwd = -c.fwd();
    bool do_air = false;
    if (c.f(F_FLIPPING)) c.setf(F_FLIPPING, c.f(F_HAS_FLIPPED) && c.flip_time < RL::FLIP_TORQUE_TIME);
    float pitch = c.ctrl[2], yaw = c.ctrl[3], roll = c.ctrl[4];
    if (c.f(F_FLIPPING)) {
        V3 rel = c.flip_rel;
        if (!is_zero(rel)) {
            float ps = 1;
            if (rel.y != 0 && pitch != 0) {
                if (rs_sgn(rel.y) == rs_sgn(pitch)) {
                    ps = 1 - rs_minf(fabsf(pitch), 1);
                    do_air = true;
                }
            }
            rel.y *= ps;
            V3 dodge = rel * V3(RL::FLIP_TORQUE_X, RL::FLIP_TORQUE_Y, 0);
            c.rb.total_torque += inverse(c.rb.inv_inertia_world) * c.rb.xf.b * dodge;
        } else {
            do_air = true;
        }
    } else {
        do_air = true;
    }
    do_air &= !c.f(F_AUTOFLIPPING);
    do_air &= update_air_control;
    if (do_air) {
        float pts = 1;
        V3 torque;
        if (pitch || yaw || roll) {
            if (c.f(F_FLIPPING)) pts = 0;
            else if (c.f(F_HAS_FLIPPED)) {
                if (c.flip_time < RL::FLIP_TORQUE_TIME + RL::FLIP_PITCHLOCK_EXTRA_TIME) pts = 0;
            }
            torque = (pitch * pitch_right * pts * RL::AIR_TORQUE_X) + (yaw * yaw_up * RL::AIR_TORQUE_Y) +
                     (roll * roll_fwd * RL::AIR_TORQUE_Z);
        } else {
            torque = V3(0, 0, 0);
        }
        V3 av = c.rb.ang_vel;
        float dp = dot(pitch_right, av) * RL::AIR_DAMP_X * (1 - fabsf(do_air ? (pitch * pts) : 0));
        float dy = dot(yaw_up, av) * RL::AIR_DAMP_Y * (1 - fabsf(do_air ? yaw : 0));
        float dr = dot(roll_fwd, av) * RL::AIR_DAMP_Z;
        V3 damping = (yaw_up * dy) + (pitch_right * dp) + (roll_fwd * dr);
        c.rb.total_torque += inverse(c.rb.inv_inertia_world) * (torque - damping) * RL::CAR_TORQUE_SCALE;
    }
    if (c.ctrl[0] != 0) c.rb.total_force += c.fwd() * c.ctrl[0] * RL::THROTTLE_AIR_ACCEL * RL::UU_TO_BT * RL::CAR_MASS_BT;
}

RSG_D void update_double_jump_or_flip(Car& c, float dt, bool pressed, float fwd_speed,
                                      const MutatorsDev& m) {  // Car.cpp:671-781
    if (c.f(F_ON_GROUND)) {
        c.setf(F_HAS_DJ, false);
        c.setf(F_HAS_FLIPPED, false);
        c.air_time = 0;
        c.air_time_sj = 0;
        c.flip_time = 0;
    } else {
        c.air_time += dt;
        if (c.f(F_HAS_JUMPED) && !c.f(F_JUMPING)) c.air_time_sj += dt;
        else c.air_time_sj = 0;
        if (pressed && c.air_time_sj < RL::DOUBLEJUMP_MAX_DELAY) {
            float pitch = c.ctrl[2], yaw = c.ctrl[3], roll = c.ctrl[4];
            float mag = fabsf(yaw) + fabsf(pitch) + fabsf(roll);
            bool flip_input = mag >= c.cfg->dodge_deadzone;
            bool can = (!c.f(F_HAS_DJ) && !c.f(F_HAS_FLIPPED)) || (flip_input ? m.unlimited_flips : m.unlimited_double_jumps);
            if (c.f(F_AUTOFLIPPING)) can = false;
            if (can) {
                if (flip_input) {
                    c.flip_time = 0;
                    c.setf(F_HAS_FLIPPED, true);
                    c.setf(F_FLIPPING, true);
                    float ratio = fabsf(fwd_speed) / RL::CAR_MAX_SPEED;
                    V3 dd(-pitch, yaw + roll, 0);
                    if (fabsf(yaw + roll) < 0.1f && fabsf(pitch) < 0.1f) dd = V3(0, 0, 0);
                    else dd = safe_normalized(dd);
                    c.flip_rel = V3(-dd.y, dd.x, 0);
                    if (fabsf(dd.x) < 0.1f) dd.x = 0;
                    if (fabsf(dd.y) < 0.1f) dd.y = 0;
                    if (!fuzzy_zero(dd)) {
                        bool back;
                        if (fabsf(fwd_speed) < 100.0f) back = dd.x < 0.0f;
                        else back = (dd.x >= 0.0f) != (fwd_speed >= 0.0f);
                        V3 iv = dd * RL::FLIP_INITIAL_VEL_SCALE;
                        float msx = back ? RL::FLIP_BACKWARD_IMPULSE_MAX_SPEED_SCALE : RL::FLIP_FORWARD_IMPULSE_MAX_SPEED_SCALE;
                        iv.x *= ((msx - 1) * ratio) + 1.f;
                        iv.y *= ((RL::FLIP_SIDE_IMPULSE_MAX_SPEED_SCALE - 1) * ratio) + 1.f;
                        if (back) iv.x *= RL::FLIP_BACKWARD_IMPULSE_SCALE_X;
                        V3 f2 = c.fwd();
                        f2.z = 0;
                        f2 = rs_normalized(f2);
                        V3 r2(-f2.y, f2.x, 0.f);
                        V3 fdv = iv.x * f2 + iv.y * r2;
                        c.rb.apply_central_impulse(fdv * RL::UU_TO_BT * RL::CAR_MASS_BT);
                    }
                } else {
                    c.rb.apply_central_impulse(c.up() * RL::JUMP_IMMEDIATE_FORCE * RL::UU_TO_BT * RL::CAR_MASS_BT);
                    c.setf(F_HAS_DJ, true);
                }
            }
        }
    }
    if (c.f(F_FLIPPING)) {
        c.flip_time += dt;
        if (c.flip_time <= RL::FLIP_TORQUE_TIME) {
            if (c.flip_time >= RL::FLIP_Z_DAMP_START && (c.rb.lin_vel.z < 0 || c.flip_time < RL::FLIP_Z_DAMP_END))
                c.rb.lin_vel.z *= powf(1 - RL::FLIP_Z_DAMP_120, dt / (1 / 120.f));
        }
    } else if (c.f(F_HAS_FLIPPED)) {
        c.flip_time += dt;
    }
}

RSG_D float roll_from_rot(const M3& m) {  // Angle::FromRotMat roll (MathTypes.cpp:62-71)
    float sp = -m.r[2].x;
    sp = sp < -1.f ? -1.f : (sp > 1.f ? 1.f : sp);
    float pitch = asinf(sp);
    float roll = atan2f(m.r[2].y, m.r[2].z);
    if (fabsf(pitch) == HALF_PI_F) {  // getEulerYPR pole case (B/LinearMath/btMatrix3x3.h:527-547)
        if (roll > 0) roll -= PI_F;
        else roll += PI_F;
    }
    return -roll;
}

RSG_D void update_auto_flip(Car& c, float dt, bool pressed) {  // Car::_UpdateAutoFlip (Car.cpp:783-817)
    if (pressed && c.f(F_WC_CONTACT) && c.wc_normal.z > RL::CAR_AUTOFLIP_NORMZ_THRESH) {
        float roll = roll_from_rot(c.rot);
        float ar = fabsf(roll);
        if (ar > RL::CAR_AUTOFLIP_ROLL_THRESH) {
            c.autoflip_timer = (float)((double)RL::CAR_AUTOFLIP_TIME * ((double)ar / 3.14159265358979323846));
            c.autoflip_scale = (roll > 0) ? 1 : -1;
            c.setf(F_AUTOFLIPPING, true);
            c.rb.apply_central_impulse(-c.up() * RL::CAR_AUTOFLIP_IMPULSE * RL::UU_TO_BT * RL::CAR_MASS_BT);
        }
    }
    if (c.f(F_AUTOFLIPPING)) {
        if (c.autoflip_timer <= 0) {
            c.setf(F_AUTOFLIPPING, false);
            c.autoflip_timer = 0;
        } else {
            c.rb.ang_vel += c.fwd() * RL::CAR_AUTOFLIP_TORQUE * c.autoflip_scale * dt;
            c.autoflip_timer -= dt;
        }
    }
}

RSG_D void update_auto_roll(Car& c, int nwc) {  // Car::_UpdateAutoRoll (Car.cpp:819-853)
    V3 gup = nwc > 0 ? upwards_from_wheels(c) : c.wc_normal;
    V3 gdown = -gup;
    V3 f = c.fwd(), r = c.right();
    V3 crossR = cross(gup, f), crossF = cross(gdown, crossR);
    float rtf = 1 - rs_clampf(dot(r, crossR), 0, 1);
    float ftf = 1 - rs_clampf(dot(f, crossF), 0, 1);
    V3 tdr = f * (dot(r, gup) >= 0 ? -1.f : 1.f);
    V3 tdf = r * (dot(f, gup) >= 0 ? 1.f : -1.f);
    c.rb.total_force += gdown * RL::CAR_AUTOROLL_FORCE * RL::UU_TO_BT * RL::CAR_MASS_BT;
    c.rb.total_torque += inverse(c.rb.inv_inertia_world) * ((tdf * ftf) + (tdr * rtf)) * RL::CAR_AUTOROLL_TORQUE;
}

RSG_D void car_set_respawn(Car& c, int idx, float boost);

// Car::_PreTickUpdate (Car.cpp:58-131) after the four suspension rays: friction, wheels, air
// control, jump, auto-flip, flip / double jump, auto-roll, suspension and boost.
// The rest of Car::_PreTickUpdate after the suspension rays (btVehicleRL::updateVehicleSecond and
// the car logic, Car.cpp:96-131), by a group of `gsize` threads of one warp (1 or 4; `wl` is the
// thread's place in it, `gmask` the group's lanes): the wheel-wise parts run one wheel per thread,
// everything that touches the whole car runs on wl == 0 in the reference's order.
RSG_DN void car_pre_after_rays_grp(const BatchView& bv, Ctx& a, Car& c, int wl, int gsize, unsigned gmask) {
#if defined(RSG_PHASE_TIMERS)
    long long ft_ = clock64();
#define RSG_FT(i) do { if (wl == 0) { long long t_ = clock64(); atomicAdd(&g_phase_cycles[i], (unsigned long long)(t_ - ft_)); ft_ = t_; } } while (0)
#else
#define RSG_FT(i)
#endif
    float dt = bv.dt;
    for (int i = wl; i < 4; i += gsize) calc_friction_impulse(a, c, dt, i);
    RSG_FT(40);
    bool pressed = c.f(F_CTRL_JUMP) && !c.f(F_LAST_JUMP);
    int nwc = 0;
    for (int i = 0; i < 4; i++) nwc += c.w[i].in_contact;
    float fwd_speed = dot(c.rb.lin_vel, c.rb.xf.b.col(0)) * RL::BT_TO_UU;
    const float hb_before = c.handbrake;
    __syncwarp(gmask);  // every thread has read the state the car part below changes
    WheelsCommon wc = update_wheels_car(c, dt, nwc, fwd_speed, hb_before, wl == 0);
    if (wl == 0) {
        for (int i = 0; i < 4; i++) c.setf(F_WHEEL0 << i, c.w[i].in_contact);
        c.setf(F_ON_GROUND, nwc >= 3);
    }
    __syncwarp(gmask);
    for (int i = wl; i < 4; i += gsize) update_wheel_friction(c, wc, i);
    __syncwarp(gmask);
    RSG_FT(41);
    if (wl == 0) {
        update_wheels_sticky(c, wc);
        if (nwc < 3) update_air_torque(c, nwc == 0);
        else c.setf(F_FLIPPING, false);
        update_jump(c, dt, pressed, bv.mut);
        update_auto_flip(c, dt, pressed);
        update_double_jump_or_flip(c, dt, pressed, fwd_speed, bv.mut);
        if (c.ctrl[0] && ((nwc > 0 && nwc < 4) || c.f(F_WC_CONTACT))) update_auto_roll(c, nwc);
        c.setf(F_WC_CONTACT, false);
    }
    RSG_FT(42);
    for (int i = wl; i < 4; i += gsize) suspension_force(c, i);
    __syncwarp(gmask);
    RSG_FT(43);
    // btVehicleRL's suspension impulses (wheels 0-3), then its friction impulses (wheels 0-3): each
    // wheel's velocity changes are computed on the wheel's thread, the first thread of the group
    // adds them to the chassis in that order (the same sums as applying the impulses one by one).
    if (gsize == 4) {
        ImpulseDeltas d = wheel_impulse_deltas(c, wl, dt);
        const int base = (threadIdx.x & 31) & ~3;
        V3 dv[4], dw[4];
        bool on[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            dv[j] = shfl_v3(gmask, d.dvs, base + j);
            dw[j] = shfl_v3(gmask, d.dws, base + j);
            on[j] = __shfl_sync(gmask, (int)d.son, base + j) != 0;
        }
        if (wl == 0)
            for (int j = 0; j < 4; j++)
                if (on[j]) { c.rb.lin_vel += dv[j]; c.rb.ang_vel += dw[j]; }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            dv[j] = shfl_v3(gmask, d.dvf, base + j);
            dw[j] = shfl_v3(gmask, d.dwf, base + j);
            on[j] = __shfl_sync(gmask, (int)d.fon, base + j) != 0;
        }
        if (wl == 0)
            for (int j = 0; j < 4; j++)
                if (on[j]) { c.rb.lin_vel += dv[j]; c.rb.ang_vel += dw[j]; }
    } else if (wl == 0) {
        apply_suspension(c, dt);
        apply_friction_impulses(c, dt);
    }
    RSG_FT(44);
    if (wl == 0) {
        update_boost(c, dt, bv.mut);
        RSG_FT(45);
    }
    __syncwarp(gmask);
}
RSG_D void car_pre_after_rays(const BatchView& bv, Ctx& a, Car& c) {
    car_pre_after_rays_grp(bv, a, c, 0, 1, 1u << (threadIdx.x & 31));
}

// Start of Car::_PreTickUpdate for a car that is not demolished and was not at the last
// pre-tick, the part of wheel `wh`: wheel 0 clamps the controls and sets the activation (nothing
// before the vehicle update reads them, and no other car's ray sees a change: the car is not and
// was not demolished), every wheel its own transform.
RSG_D void car_pre_before_rays_wheel(Car& c, int wh) {
    if (wh == 0) {
        for (int k = 0; k < 5; k++) c.ctrl[k] = rs_clampf(c.ctrl[k], -1, 1);
        c.rb.act = ACTIVE_TAG;
        c.rb.no_contact_response = false;
    }
    update_wheel_transform(c, wh);
}

RSG_DN void car_pre_tick(const BatchView& bv, Ctx& a, Car& c) {  // Car::_PreTickUpdate (Car.cpp:58-131)
    float dt = bv.dt;
    for (int k = 0; k < 5; k++) c.ctrl[k] = rs_clampf(c.ctrl[k], -1, 1);
    if (c.f(F_DEMOED)) {
        c.demo_timer = rs_maxf(c.demo_timer - dt, 0);
        if (c.demo_timer == 0) car_set_respawn(c, 0, bv.mut.car_spawn_boost);
        c.rb.act = DISABLE_SIMULATION;
        c.rb.no_contact_response = true;
    } else {
        c.rb.act = ACTIVE_TAG;
        c.rb.no_contact_response = false;
    }
    if (c.f(F_DEMOED)) return;
    for (int i = 0; i < 4; i++) update_wheel_transform(c, i);
    for (int i = 0; i < 4; i++) ray_cast_wheel(bv, a, c, i);
    car_pre_after_rays(bv, a, c);
}

RSG_D void car_post_tick(Car& c, float dt) {  // Car::_PostTickUpdate (Car.cpp:133-163)
    if (c.f(F_DEMOED)) return;
    c.rot = c.rb.xf.b;
    float sp2 = len2(c.rb.lin_vel * RL::BT_TO_UU);
    bool ss;
    if (c.f(F_SUPERSONIC) && c.supersonic_time < RL::SUPERSONIC_MAINTAIN_MAX_TIME)
        ss = (sp2 >= RL::SUPERSONIC_MAINTAIN_MIN_SPEED * RL::SUPERSONIC_MAINTAIN_MIN_SPEED);
    else
        ss = (sp2 >= RL::SUPERSONIC_START_SPEED * RL::SUPERSONIC_START_SPEED);
    c.setf(F_SUPERSONIC, ss);
    if (ss) c.supersonic_time += dt;
    else c.supersonic_time = 0;
    if (c.cc_cooldown > 0) c.cc_cooldown = rs_maxf(c.cc_cooldown - dt, 0);
    for (int k = 0; k < 5; k++) c.last_ctrl[k] = c.ctrl[k];
    c.setf(F_LAST_JUMP, c.f(F_CTRL_JUMP));
    c.setf(F_LAST_BOOST, c.f(F_CTRL_BOOST));
    c.setf(F_LAST_HB, c.f(F_CTRL_HB));
}

RSG_D void car_finish_physics(Car& c) {  // Car::_FinishPhysicsTick (Car.cpp:165-193)
    if (c.f(F_DEMOED)) return;
    if (!is_zero(c.vel_cache)) {
        c.rb.lin_vel += c.vel_cache;
        c.vel_cache = V3(0, 0, 0);
    }
    V3 v = c.rb.lin_vel, w = c.rb.ang_vel;
    const float ms = RL::CAR_MAX_SPEED * RL::UU_TO_BT;
    if (len2(v) > ms * ms) v = normalized(v) * ms;
    if (len2(w) > (RL::CAR_MAX_ANG_SPEED * RL::CAR_MAX_ANG_SPEED)) w = normalized(w) * RL::CAR_MAX_ANG_SPEED;
    c.rb.lin_vel = v;
    c.rb.ang_vel = w;
    c.ticks_since++;
}

RSG_D void car_set_respawn(Car& c, int idx, float boost) {  // Car::Respawn (Car.cpp:43-56) + SetState
    float team_sign = c.f(F_TEAM_ORANGE) ? -1.f : 1.f;
    V3 pos(c_respawn_locs[idx][0], c_respawn_locs[idx][1] * team_sign, RL::CAR_RESPAWN_Z);
    float yaw = (float)((double)(float)(3.14159265358979323846 / 2) + (c.f(F_TEAM_ORANGE) ? 3.14159265358979323846 : 0));
    M3 m = m_euler_ypr(yaw, -0.f, -0.f);
    c.rb.xf.o = pos * RL::UU_TO_BT;
    c.rb.xf.b = m;
    c.rb.lin_vel = V3(0, 0, 0);
    c.rb.ang_vel = V3(0, 0, 0);
    c.rb.update_inertia();
    c.vel_cache = V3(0, 0, 0);
    c.rot = m;
    uint32_t keep = c.flags & (F_PRESENT | F_TEAM_ORANGE | F_CTRL_JUMP | F_CTRL_BOOST | F_CTRL_HB);
    c.flags = keep | F_ON_GROUND;
    c.flip_rel = V3(0, 0, 0);
    c.jump_time = c.flip_time = c.air_time = c.air_time_sj = 0;
    c.boost = boost;
    c.time_since_boost = c.boosting_time = c.supersonic_time = c.handbrake = 0;
    c.autoflip_timer = c.autoflip_scale = 0;
    c.wc_normal = V3(0, 0, 0);
    c.cc_other = 0;
    c.cc_cooldown = 0;
    c.demo_timer = 0;
    c.bhi_rel = c.bhi_ballpos = c.bhi_extra = V3(0, 0, 0);
    c.bhi_hit = ~0ull;
    c.bhi_extra_tick = ~0ull;
    c.ticks_since = 0;
    for (int k = 0; k < 5; k++) c.last_ctrl[k] = 0;
}


// ---------------------------------------------------------------- shapes / AABBs
RSG_D void car_box_aabb(const Car& c, const Xf& child, V3& mn, V3& mx) { transform_aabb(car_he(c), c.cfg->margin, child, mn, mx); }
RSG_D void car_compound_aabb(const Car& c, const Xf& t, V3& mn, V3& mx) {  // btCompoundShape::getAabb
    V3 cmin(c.cfg->comp_min[0], c.cfg->comp_min[1], c.cfg->comp_min[2]);
    V3 cmax(c.cfg->comp_max[0], c.cfg->comp_max[1], c.cfg->comp_max[2]);
    V3 lhe = 0.5f * (cmax - cmin);
    V3 lc = 0.5f * (cmax + cmin);
    M3 ab = absolute(t.b);
    V3 center = xf_apply(t, lc);
    V3 ext(dot(ab.r[0], lhe), dot(ab.r[1], lhe), dot(ab.r[2], lhe));
    mn = center - ext;
    mx = center + ext;
}
RSG_D void ball_aabb(const Xf& t, float radius, V3& mn, V3& mx) {
    float m = radius + 0.08f;
    mn = t.o - V3(m, m, m);
    mx = t.o + V3(m, m, m);
}
RSG_D void mesh_aabb(const DevMesh& m, V3& mn, V3& mx) {  // btTriangleMeshShape::getAabb, identity transform
    V3 lhe = 0.5f * (m.aabb_max - m.aabb_min);
    V3 lc = 0.5f * (m.aabb_max + m.aabb_min);
    mn = lc - lhe;
    mx = lc + lhe;
}

// btTransformUtil::integrateTransform (B/LinearMath/btTransformUtil.h:37-80)
RSG_D void integrate_transform(const Xf& cur, V3 lv, V3 av, float dt, bool no_rot, Xf& out) {
    out.o = cur.o + lv * dt;
    if (no_rot) { out.b = cur.b; return; }
    const float ANGULAR_MOTION_THRESHOLD = 0.5f * HALF_PI_F;
    float a2 = len2(av);
    float ang = 0;
    if (a2 > SIMD_EPS) ang = sqrtf(a2);
    if (ang * dt > ANGULAR_MOTION_THRESHOLD) ang = ANGULAR_MOTION_THRESHOLD / dt;
    V3 axis;
    if (ang < 0.001f) axis = av * (0.5f * dt - (dt * dt * dt) * (0.020833333333f) * ang * ang);
    else axis = av * (sinf(0.5f * ang * dt) / ang);
    Q dorn(axis.x, axis.y, axis.z, cosf(ang * dt * 0.5f));
    Q orn0 = q_from_m(cur.b);
    Q pred = q_safe_normalize(q_mul(dorn, orn0));
    if (q_len2(pred) > SIMD_EPS) out.b = m_from_q(pred);
    else out.b = cur.b;
}

// ---------------------------------------------------------------- contact manifolds
// btManifoldResult::addContactPoint (B/.../CollisionDispatch/btManifoldResult.cpp:109-194)
RSG_D int add_point(Ctx& a, Manifold& m, const Xf& x0, const Xf& x1, V3 n, V3 pb, float depth, float friction,
                    float restitution) {
    if (depth > m.breaking) return -1;
    V3 pa = pb + n * depth;
    MPoint p;
    p.local_a = xf_inv_apply(x0, pa);
    p.local_b = xf_inv_apply(x1, pb);
    p.normal = n;
    p.dist = depth;
    p.pos_a = pa;
    p.pos_b = pb;
    p.friction = friction;
    p.restitution = restitution;
    p.special = false;
    int idx;
    if (m.n == 4) {
        // btPersistentManifold::sortCachedPoints (btPersistentManifold.cpp:113-190)
        int maxPen = -1;
        float maxv = p.dist;
        for (int i = 0; i < 4; i++)
            if (a.pts[m.pt[i]].dist < maxv) { maxPen = i; maxv = a.pts[m.pt[i]].dist; }
        V3 l0 = a.pts[m.pt[0]].local_a, l1 = a.pts[m.pt[1]].local_a, l2 = a.pts[m.pt[2]].local_a, l3 = a.pts[m.pt[3]].local_a;
        float r0 = 0, r1 = 0, r2 = 0, r3 = 0;
        if (maxPen != 0) r0 = len2(cross(p.local_a - l1, l3 - l2));
        if (maxPen != 1) r1 = len2(cross(p.local_a - l0, l3 - l2));
        if (maxPen != 2) r2 = len2(cross(p.local_a - l0, l3 - l1));
        if (maxPen != 3) r3 = len2(cross(p.local_a - l0, l2 - l1));
        idx = closest_axis4(r0, r1, r2, r3);
        if (idx < 0) idx = 0;
    } else {
        if (a.npts >= a.cap_pts) {
            a.err |= ERR_POINT_OVERFLOW;
            return -1;
        }
        idx = m.n++;
        m.pt[idx] = (int8_t)a.npts++;
    }
    a.pts[m.pt[idx]] = p;
    return idx;
}

// btPersistentManifold::refreshContactPoints (btPersistentManifold.cpp:263-318)
RSG_D void refresh(Ctx& a, Manifold& m, const Xf& x0, const Xf& x1) {
    for (int i = m.n - 1; i >= 0; i--) {
        MPoint& p = a.pts[m.pt[i]];
        p.pos_a = xf_apply(x0, p.local_a);
        p.pos_b = xf_apply(x1, p.local_b);
        p.dist = dot(p.pos_a - p.pos_b, p.normal);
    }
    for (int i = m.n - 1; i >= 0; i--) {
        MPoint& p = a.pts[m.pt[i]];
        bool remove = false;
        if (!(p.dist <= m.breaking)) remove = true;
        else {
            V3 proj = p.pos_a - p.normal * p.dist;
            V3 diff = p.pos_b - proj;
            if (dot(diff, diff) > m.breaking * m.breaking) remove = true;
        }
        if (remove) {
            int last = m.n - 1;
            if (i != last) m.pt[i] = m.pt[last];
            m.n--;
        }
    }
}

// btAdjustInternalEdgeContacts (B/.../CollisionDispatch/btInternalEdgeUtility.cpp:414-840) for a
// mesh triangle contact; the mesh transform is the identity and the flags argument is 0.
RSG_D void nearest_on_segment(V3 p, V3 l0, V3 l1, V3& out) {
    V3 d = l1 - l0;
    if (fuzzy_zero(d)) { out = l0; return; }
    float t = dot(p - l0, d) / dot(d, d);
    if (t < 0) t = 0;
    else if (t > 1) t = 1;
    out = l0 + d * t;
}
RSG_D bool clamp_normal(V3 edge, V3 tri_n, V3 local_n, float corrected, V3& out) {
    V3 ec = normalized(cross(edge, tri_n));
    float cur = atan2f(dot(local_n, ec), dot(local_n, tri_n));
    if (corrected < 0) {
        if (cur < corrected) {
            out = m_from_q(q_axis_angle(edge, corrected - cur)) * local_n;
            return true;
        }
    }
    if (corrected >= 0) {
        if (cur > corrected) {
            out = m_from_q(q_axis_angle(edge, corrected - cur)) * local_n;
            return true;
        }
    }
    return false;
}
RSG_D void edge_case(MPoint& cp, const TriInfo& inf, V3 tri_n, V3 lcn, V3 edge, float angle, int convflag,
                     int swapflag, bool recompute_local, bool& near_edge, int& concave) {
    near_edge = true;
    if (angle == 0.f) { concave++; return; }
    bool conv = (inf.flags & convflag) != 0;
    float sf = conv ? 1.f : -1.f;
    V3 nA = sf * tri_n;
    V3 cnB = q_rotate(q_axis_angle(edge, angle), tri_n);
    if (inf.flags & swapflag) cnB *= -1;
    V3 nB = sf * cnB;
    float ndA = dot(lcn, nA), ndB = dot(lcn, nB);
    if ((ndA < 0.f) && (ndB < 0.f)) { concave++; return; }
    V3 ln = recompute_local ? cp.normal : lcn;
    V3 clamped;
    if (clamp_normal(edge, sf * tri_n, ln, angle, clamped)) {
        if (dot(clamped, tri_n) > 0) {
            cp.normal = clamped;
            cp.pos_b = cp.pos_a - cp.normal * cp.dist;
            cp.local_b = cp.pos_b;
        }
    }
}
RSG_DN void adjust_internal_edge(const DevMesh& mesh, MPoint& cp, int tri) {
    TriInfo inf = mesh.info[tri];
    if (!inf.present) return;
    V3 v[3];
    tri_load(mesh, tri, v);
    V3 tri_n = normalized(cross(v[1] - v[0], v[2] - v[0]));
    V3 nearest;
    nearest_on_segment(cp.local_b, v[0], v[1], nearest);
    V3 contact = cp.local_b;
    bool near_edge = false;
    int concave = 0;
    V3 lcn = normalized(cp.normal);
    int best = -1;
    float bestd = BT_LARGE;
    const float MAXA = TWO_PI_F, EDGE_D = 0.1f;
    if (fabsf(inf.a01) < MAXA) {
        V3 nn; nearest_on_segment(cp.local_b, v[0], v[1], nn);
        float l = len(contact - nn);
        if (l < bestd) { best = 0; bestd = l; }
    }
    if (fabsf(inf.a12) < MAXA) {
        V3 nn; nearest_on_segment(cp.local_b, v[1], v[2], nn);
        float l = len(contact - nn);
        if (l < bestd) { best = 1; bestd = l; }
    }
    if (fabsf(inf.a20) < MAXA) {
        V3 nn; nearest_on_segment(cp.local_b, v[2], v[0], nn);
        float l = len(contact - nn);
        if (l < bestd) { best = 2; bestd = l; }
    }
    if (fabsf(inf.a01) < MAXA) {
        float l = len(contact - nearest);
        if (l < EDGE_D && best == 0)
            edge_case(cp, inf, tri_n, lcn, v[0] - v[1], inf.a01, TRI_V0V1_CONVEX, TRI_V0V1_SWAP, false, near_edge, concave);
    }
    nearest_on_segment(contact, v[1], v[2], nearest);
    if (fabsf(inf.a12) < MAXA) {
        float l = len(contact - nearest);
        if (l < EDGE_D && best == 1)
            edge_case(cp, inf, tri_n, lcn, v[1] - v[2], inf.a12, TRI_V1V2_CONVEX, TRI_V1V2_SWAP, true, near_edge, concave);
    }
    nearest_on_segment(contact, v[2], v[0], nearest);
    if (fabsf(inf.a20) < MAXA) {
        float l = len(contact - nearest);
        if (l < EDGE_D && best == 2)
            edge_case(cp, inf, tri_n, lcn, v[2] - v[0], inf.a20, TRI_V2V0_CONVEX, TRI_V2V0_SWAP, true, near_edge, concave);
    }
    if (near_edge && concave > 0) {
        if (dot(tri_n, lcn) < 0) return;
        cp.normal = tri_n;
        cp.pos_b = cp.pos_a - cp.normal * cp.dist;
        cp.local_b = cp.pos_b;
    }
}

// ---------------------------------------------------------------- GJK
// btGjkPairDetector::getClosestPointsNonVirtual (B/.../NarrowPhaseCollision/btGjkPairDetector.cpp:693-959)
// with btVoronoiSimplexSolver (btVoronoiSimplexSolver.cpp)
struct Convex {
    int type;  // 0 box (implicit half extents he), 1 sphere (point core), 2 triangle
    V3 he;
    V3 tv[3];
    float margin;
    RSG_D V3 support_nomargin(V3 d) const {
        if (type == 0) return V3(d.x >= 0 ? he.x : -he.x, d.y >= 0 ? he.y : -he.y, d.z >= 0 ? he.z : -he.z);
        if (type == 1) return V3(0, 0, 0);
        V3 dots(dot(d, tv[0]), dot(d, tv[1]), dot(d, tv[2]));
        return tv[max_axis(dots)];
    }
    RSG_D void aabb(const Xf& t, V3& mn, V3& mx) const {
        if (type == 0) { transform_aabb(he, margin, t, mn, mx); return; }
        if (type == 1) {
            float m = margin + 0.08f;
            mn = t.o - V3(m, m, m);
            mx = t.o + V3(m, m, m);
            return;
        }
        V3 a(BT_LARGE, BT_LARGE, BT_LARGE), b(-BT_LARGE, -BT_LARGE, -BT_LARGE);
        for (int i = 0; i < 3; i++) {
            V3 w = xf_apply(t, tv[i]);
            a = vmin(a, w);
            b = vmax(b, w);
        }
        mn = a - V3(margin, margin, margin);
        mx = b + V3(margin, margin, margin);
    }
};

struct SubResult {
    V3 closest;
    bool used[4];
    float bary[4];
    bool degenerate;
    RSG_D void reset() {
        degenerate = false;
        for (int i = 0; i < 4; i++) { used[i] = false; bary[i] = 0; }
    }
    RSG_D bool valid() const { return bary[0] >= 0 && bary[1] >= 0 && bary[2] >= 0 && bary[3] >= 0; }
    RSG_D void set_bary(float a, float b, float c, float d) { bary[0] = a; bary[1] = b; bary[2] = c; bary[3] = d; }
};

RSG_D void closest_tri(V3 p, V3 a, V3 b, V3 c, SubResult& r) {  // closestPtPointTriangle
    r.used[0] = r.used[1] = r.used[2] = r.used[3] = false;
    V3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) { r.closest = a; r.used[0] = true; r.set_bary(1, 0, 0, 0); return; }
    V3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) { r.closest = b; r.used[1] = true; r.set_bary(0, 1, 0, 0); return; }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
        float v = d1 / (d1 - d3);
        r.closest = a + v * ab; r.used[0] = r.used[1] = true; r.set_bary(1 - v, v, 0, 0);
        return;
    }
    V3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.f && d5 <= d6) { r.closest = c; r.used[2] = true; r.set_bary(0, 0, 1, 0); return; }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
        float w = d2 / (d2 - d6);
        r.closest = a + w * ac; r.used[0] = r.used[2] = true; r.set_bary(1 - w, 0, w, 0);
        return;
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        r.closest = b + w * (c - b); r.used[1] = r.used[2] = true; r.set_bary(0, 1 - w, w, 0);
        return;
    }
    float denom = 1.f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    r.closest = a + ab * v + ac * w;
    r.used[0] = r.used[1] = r.used[2] = true;
    r.set_bary(1 - v - w, v, w, 0);
}
RSG_D int point_outside(V3 p, V3 a, V3 b, V3 c, V3 d) {  // pointOutsideOfPlane
    V3 nrm = cross(b - a, c - a);
    float sp = dot(p - a, nrm), sd = dot(d - a, nrm);
    if (sd * sd < (1e-4f * 1e-4f)) return -1;
    return sp * sd < 0.f;
}
RSG_DN bool closest_tet(V3 p, V3 a, V3 b, V3 c, V3 d, SubResult& fr) {  // closestPtPointTetrahedron
    SubResult t;
    t.reset();
    fr.closest = p;
    fr.used[0] = fr.used[1] = fr.used[2] = fr.used[3] = true;
    int oABC = point_outside(p, a, b, c, d), oACD = point_outside(p, a, c, d, b), oADB = point_outside(p, a, d, b, c),
        oBDC = point_outside(p, b, d, c, a);
    if (oABC < 0 || oACD < 0 || oADB < 0 || oBDC < 0) { fr.degenerate = true; return false; }
    if (!oABC && !oACD && !oADB && !oBDC) return false;
    float best = FLT_MAX;
    if (oABC) {
        closest_tri(p, a, b, c, t);
        V3 q = t.closest;
        float sq = dot(q - p, q - p);
        if (sq < best) {
            best = sq; fr.closest = q;
            fr.used[0] = t.used[0]; fr.used[1] = t.used[1]; fr.used[2] = t.used[2]; fr.used[3] = false;
            fr.set_bary(t.bary[0], t.bary[1], t.bary[2], 0);
        }
    }
    if (oACD) {
        closest_tri(p, a, c, d, t);
        V3 q = t.closest;
        float sq = dot(q - p, q - p);
        if (sq < best) {
            best = sq; fr.closest = q;
            fr.used[0] = t.used[0]; fr.used[1] = false; fr.used[2] = t.used[1]; fr.used[3] = t.used[2];
            fr.set_bary(t.bary[0], 0, t.bary[1], t.bary[2]);
        }
    }
    if (oADB) {
        closest_tri(p, a, d, b, t);
        V3 q = t.closest;
        float sq = dot(q - p, q - p);
        if (sq < best) {
            best = sq; fr.closest = q;
            fr.used[0] = t.used[0]; fr.used[1] = t.used[2]; fr.used[2] = false; fr.used[3] = t.used[1];
            fr.set_bary(t.bary[0], t.bary[2], 0, t.bary[1]);
        }
    }
    if (oBDC) {
        closest_tri(p, b, d, c, t);
        V3 q = t.closest;
        float sq = dot(q - p, q - p);
        if (sq < best) {
            best = sq; fr.closest = q;
            fr.used[0] = false; fr.used[1] = t.used[0]; fr.used[2] = t.used[2]; fr.used[3] = t.used[1];
            fr.set_bary(0, t.bary[0], t.bary[2], t.bary[1]);
        }
    }
    return true;
}

struct Simplex {
    int n;
    V3 W[5], Pp[5], Qq[5];
    V3 lastW;
    bool needs_update, cached_valid;
    V3 cP1, cP2, cV;
    SubResult bc;
    RSG_D void reset() {
        cached_valid = false;
        n = 0;
        needs_update = true;
        lastW = V3(BT_LARGE, BT_LARGE, BT_LARGE);
        bc.reset();
    }
    RSG_D void remove(int i) {
        n--;
        W[i] = W[n]; Pp[i] = Pp[n]; Qq[i] = Qq[n];
    }
    RSG_D void reduce(const SubResult& r) {
        if (n >= 4 && !r.used[3]) remove(3);
        if (n >= 3 && !r.used[2]) remove(2);
        if (n >= 2 && !r.used[1]) remove(1);
        if (n >= 1 && !r.used[0]) remove(0);
    }
    RSG_D void add(V3 w, V3 p, V3 q) {
        lastW = w;
        needs_update = true;
        W[n] = w; Pp[n] = p; Qq[n] = q;
        n++;
    }
    RSG_D bool update() {
        if (!needs_update) return cached_valid;
        bc.reset();
        needs_update = false;
        V3 p(0, 0, 0);
        switch (n) {
            case 0: cached_valid = false; break;
            case 1:
                cP1 = Pp[0]; cP2 = Qq[0]; cV = cP1 - cP2;
                bc.reset(); bc.set_bary(1, 0, 0, 0);
                cached_valid = bc.valid();
                break;
            case 2: {
                V3 from = W[0], to = W[1];
                V3 diff = p - from, v = to - from;
                float t = dot(v, diff);
                if (t > 0) {
                    float vv = dot(v, v);
                    if (t < vv) { t /= vv; bc.used[0] = bc.used[1] = true; }
                    else { t = 1; bc.used[1] = true; }
                } else {
                    t = 0;
                    bc.used[0] = true;
                }
                bc.set_bary(1 - t, t, 0, 0);
                cP1 = Pp[0] + t * (Pp[1] - Pp[0]);
                cP2 = Qq[0] + t * (Qq[1] - Qq[0]);
                cV = cP1 - cP2;
                reduce(bc);
                cached_valid = bc.valid();
                break;
            }
            case 3: {
                closest_tri(p, W[0], W[1], W[2], bc);
                cP1 = Pp[0] * bc.bary[0] + Pp[1] * bc.bary[1] + Pp[2] * bc.bary[2];
                cP2 = Qq[0] * bc.bary[0] + Qq[1] * bc.bary[1] + Qq[2] * bc.bary[2];
                cV = cP1 - cP2;
                reduce(bc);
                cached_valid = bc.valid();
                break;
            }
            case 4: {
                bool sep = closest_tet(p, W[0], W[1], W[2], W[3], bc);
                if (sep) {
                    cP1 = Pp[0] * bc.bary[0] + Pp[1] * bc.bary[1] + Pp[2] * bc.bary[2] + Pp[3] * bc.bary[3];
                    cP2 = Qq[0] * bc.bary[0] + Qq[1] * bc.bary[1] + Qq[2] * bc.bary[2] + Qq[3] * bc.bary[3];
                    cV = cP1 - cP2;
                    reduce(bc);
                } else {
                    if (bc.degenerate) cached_valid = false;
                    else { cached_valid = true; cV = V3(0, 0, 0); }
                    break;
                }
                cached_valid = bc.valid();
                break;
            }
            default: cached_valid = false;
        }
        return cached_valid;
    }
    RSG_D bool closest(V3& v) { bool ok = update(); v = cV; return ok; }
    RSG_D bool in_simplex(V3 w) const {
        bool found = false;
        for (int i = 0; i < n; i++)
            if (len2(W[i] - w) <= 0.0001f) { found = true; break; }
        if (w == lastW) return true;
        return found;
    }
    RSG_D void points(V3& p1, V3& p2) { update(); p1 = cP1; p2 = cP2; }
};

}  // namespace rsg
#include "rsg_epa.cuh"
namespace rsg {

// btSubsimplexConvexCast::calcTimeOfImpact (B/BulletCollision/NarrowPhaseCollision/btSubSimplexConvexCast.cpp:30-141)
// of a point (btSphereShape of radius and margin 0, btCollisionWorld.cpp:271-273) moving from `from`
// to `to` against a static convex shape with world support vertex `support(d, o)` for its origin at o,
// then the acceptance of btCollisionWorld::rayTestSingleInternal (btCollisionWorld.cpp:288-310): a
// normal longer than 0.01 and a fraction below the closest hit so far.  The shape's transform is
// interpolated like the point's (btSubSimplexConvexCast.cpp:93-94), between two equal origins, which
// moves it by rounding.  32 iterations, epsilon 1e-4 (btConvexCast.h:28-29),
// no allowed penetration; the point's supporting vertex is its origin.
template <class Sup>
RSG_D bool ray_subsimplex(V3 from, V3 to, V3 ob, Sup support, float& hit_frac, V3& out_n) {
    Simplex sx;
    sx.reset();
    V3 r = to - from;
    float lambda = 0.f;
    V3 xa = from, xb = ob;
    V3 sa = xa, sb = support(r, ob);
    V3 v = sa - sb;
    int max_iter = 32;
    V3 n(0, 0, 0);
    float dist2 = len2(v);
    V3 w;
    while ((dist2 > 0.0001f) && max_iter--) {
        sa = xa;
        sb = support(v, xb);
        w = sa - sb;
        float vdw = dot(v, w);
        if (lambda > 1.f) return false;
        if (vdw > 0.f) {
            float vdr = dot(v, r);
            if (vdr >= -(SIMD_EPS * SIMD_EPS)) return false;
            lambda = lambda - vdw / vdr;
            xa = lerp(from, to, lambda);
            xb = lerp(ob, ob, lambda);
            w = sa - sb;
            n = v;
        }
        if (!sx.in_simplex(w)) sx.add(w, sa, sb);
        if (sx.closest(v)) dist2 = len2(v);
        else dist2 = 0.f;
    }
    V3 nrm = len2(n) >= (SIMD_EPS * SIMD_EPS) ? normalized(n) : V3(0, 0, 0);
    if (dot(nrm, r) >= -0.f) return false;
    if (!(len2(nrm) > 0.0001f)) return false;
    if (!(lambda < hit_frac)) return false;
    hit_frac = lambda;
    out_n = normalized(nrm);
    return true;
}

// btBoxShape::localGetSupportingVertex (btBoxShape.h:47-56) with the margin in the half extents
RSG_DN bool ray_cast_box(V3 from, V3 to, const Xf& box_xf, V3 he_margin, float& hit_frac, V3& out_n) {
    auto sup = [&](V3 d, V3 o) {
        V3 l = d * box_xf.b;
        V3 s(l.x >= 0.f ? he_margin.x : -he_margin.x, l.y >= 0.f ? he_margin.y : -he_margin.y,
             l.z >= 0.f ? he_margin.z : -he_margin.z);
        Xf t = box_xf;
        t.o = o;
        return xf_apply(t, s);
    };
    return ray_subsimplex(from, to, box_xf.o, sup, hit_frac, out_n);
}

// btSphereShape::localGetSupportingVertex (btSphereShape.cpp:37-49): the margin (the radius) along the
// normalised direction, (-1,-1,-1) normalised for a vanishing one
RSG_DN bool ray_cast_sphere(V3 from, V3 to, const Xf& xf, float radius, float& hit_frac, V3& out_n) {
    auto sup = [&](V3 d, V3 o) {
        V3 l = d * xf.b;
        if (len2(l) < (SIMD_EPS * SIMD_EPS)) l = normalized(V3(-1, -1, -1));
        else l = normalized(l);
        Xf t = xf;
        t.o = o;
        return xf_apply(t, l * radius);
    };
    return ray_subsimplex(from, to, xf.o, sup, hit_frac, out_n);
}

struct GjkOut {
    bool valid;
    V3 normal, point_on_b;
    float dist;
    bool epa_needed;  // the pair needed EPA and no work slot was free (WARN_EPA_SKIPPED)
};

RSG_DN GjkOut gjk(const Convex& A, const Xf& ta_in, const Convex& B, const Xf& tb_in, float max_dist2) {
    GjkOut out;
    out.valid = false;
    out.epa_needed = false;
    out.dist = 0;
    float distance = 0;
    V3 normalInB(0, 0, 0), pA, pB;
    Xf ta = ta_in, tb = tb_in;
    V3 off = (ta.o + tb.o) * 0.5f;
    ta.o -= off;
    tb.o -= off;
    float mA = A.margin, mB = B.margin;
    V3 sep(0, 1, 0);
    bool is_valid = false, check_simplex = false;
    int degenerate = 0;
    Simplex sx;
    sx.reset();
    float sqd = BT_LARGE, delta = 0, margin = mA + mB;
    int iter = 0;
    while (true) {
        V3 sa = (-sep) * ta_in.b;
        V3 sb = sep * tb_in.b;
        V3 pin = A.support_nomargin(sa), qin = B.support_nomargin(sb);
        V3 pw = xf_apply(ta, pin), qw = xf_apply(tb, qin);
        V3 w = pw - qw;
        delta = dot(sep, w);
        if ((delta > 0.f) && (delta * delta > sqd * max_dist2)) { degenerate = 10; check_simplex = true; break; }
        if (sx.in_simplex(w)) { degenerate = 1; check_simplex = true; break; }
        float f0 = sqd - delta, f1 = sqd * 1.0e-6f;
        if (f0 <= f1) { degenerate = f0 <= 0.f ? 2 : 11; check_simplex = true; break; }
        sx.add(w, pw, qw);
        V3 nsep;
        if (!sx.closest(nsep)) { degenerate = 3; check_simplex = true; break; }
        if (len2(nsep) < 1.0e-6f) { sep = nsep; degenerate = 6; check_simplex = true; break; }
        float prev = sqd;
        sqd = len2(nsep);
        if (prev - sqd <= SIMD_EPS * prev) { check_simplex = true; degenerate = 12; break; }
        sep = nsep;
        if (iter++ > 1000) break;
        if (sx.n == 4) { degenerate = 13; break; }
    }
    if (check_simplex) {
        sx.points(pA, pB);
        normalInB = sep;
        float l2 = len2(sep);
        if (l2 < 0.0001f) degenerate = 5;
        if (l2 > SIMD_EPS * SIMD_EPS) {
            float rlen = 1.f / sqrtf(l2);
            normalInB *= rlen;
            float s = sqrtf(sqd);
            pA -= sep * (mA / s);
            pB += sep * (mB / s);
            distance = ((1.f / rlen) - margin);
            is_valid = true;
        }
    }
    bool catch_deg = degenerate && ((distance + margin) < 0.01f);
    if (!is_valid || catch_deg) {
        // penetration depth (btGjkPairDetector.cpp:850-922)
        const int slot = epa::acquire_slot();
        if (slot < 0) {
            out.epa_needed = true;
            if (!is_valid) return out;
        } else {
            V3 sep_axis(0, 0, 0), tA, tB;
            const bool valid2 = epa::calc_pen_depth(A, ta, B, tb, epa::g_epa_slots + slot, sep_axis, tA, tB);
            epa::release_slot(slot);
            if (valid2) {
                V3 tn = tB - tA;
                float l2 = len2(tn);
                if (l2 <= SIMD_EPS * SIMD_EPS) {
                    tn = sep_axis;
                    l2 = len2(sep_axis);
                }
                if (l2 > SIMD_EPS * SIMD_EPS) {
                    tn = tn / sqrtf(l2);
                    const float d2 = -len(tA - tB);
                    if (!is_valid || (d2 < distance)) {
                        distance = d2;
                        pA = tA;
                        pB = tB;
                        normalInB = tn;
                        is_valid = true;
                    }
                }
            } else if (len2(sep_axis) > 0.f) {
                const float d2 = len(tA - tB) - margin;
                if (!is_valid || (d2 < distance)) {
                    distance = d2;
                    pA = tA - sep_axis * mA;
                    pB = tB + sep_axis * mB;
                    normalInB = normalized(sep_axis);
                    is_valid = true;
                }
            }
            if (!is_valid) return out;
        }
    }
    if (is_valid && ((distance < 0) || (distance * distance < max_dist2))) {
        V3 amn, amx, bmn, bmx;  // m_fixContactNormalDirection
        A.aabb(ta, amn, amx);
        B.aabb(tb, bmn, bmx);
        V3 posA = (amx + amn) * 0.5f, posB = (bmn + bmx) * 0.5f;
        if (dot(posA - posB, normalInB) < 0.f) normalInB *= -1.f;
        out.valid = true;
        out.normal = normalInB;
        out.point_on_b = pB + off;
        out.dist = distance;
    }
    return out;
}

// closestPointTriangle (B/.../CollisionDispatch/SphereTriangleDetector.cpp:87-128): vertex
// regions are tested before edge regions, unlike the simplex solver's variant above
RSG_D V3 closest_point_triangle(V3 p, V3 a, V3 b, V3 c) {
    V3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) return a;
    V3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) return b;
    V3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.f && d5 <= d6) return c;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) return a + (d1 / (d1 - d3)) * ab;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) return a + (d2 / (d2 - d6)) * ac;
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) return b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
    float denom = 1.f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    return a + v * ab + w * ac;
}

// SphereTriangleDetector::collide (B/.../CollisionDispatch/SphereTriangleDetector.cpp:139-281)
RSG_DN bool sphere_triangle(V3 center, float radius, const V3 v[3], float threshold, V3& point, V3& normal_out,
                            float& depth) {
    float rwt = radius + threshold;
    V3 n = cross(v[1] - v[0], v[2] - v[0]);
    float l2 = len2(n);
    bool has = false;
    V3 cpnt;
    if (l2 >= SIMD_EPS * SIMD_EPS) {
        n = n / sqrtf(l2);
        V3 p1c = center - v[0];
        float dfp = dot(p1c, n);
        if (dfp < 0.f) { dfp *= -1.f; n *= -1.f; }
        if (dfp < rwt) {
            V3 u = v[1] - v[0], vv = v[2] - v[0];
            V3 nn = cross(u, vv);
            float nl = dot(nn, nn);
            V3 w = center - v[0];
            float gamma = dot(cross(u, w), nn) / nl;
            float beta = dot(cross(w, vv), nn) / nl;
            float alpha = 1 - gamma - beta;
            bool inside = (0 <= alpha) && (alpha <= 1) && (0 <= beta) && (beta <= 1) && (0 <= gamma) && (gamma <= 1);
            if (inside) {
                has = true;
                cpnt = center - n * dfp;
            } else {
                V3 res = closest_point_triangle(center, v[0], v[1], v[2]);
                float dsq = len2(res - center);
                if (dsq < rwt * rwt) { has = true; cpnt = res; }
            }
        }
    }
    if (has) {
        V3 c2 = center - cpnt;
        float dsq = len2(c2);
        if (dsq < rwt * rwt) {
            if (dsq > SIMD_EPS) {
                float d = sqrtf(dsq);
                normal_out = normalized(c2);
                point = cpnt;
                depth = -(radius - d);
            } else {
                normal_out = n;
                point = cpnt;
                depth = -radius;
            }
            return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------- box-box
// btBoxBoxDetector (B/.../CollisionDispatch/btBoxBoxDetector.cpp:30-767): the separating-axis
// test between two car boxes and its contact clipping, in the reference's operation order.
struct BoxHit {
    V3 point;
    float depth;
};
RSG_D float col_dot(const M3& m, int j, V3 v) { return m.r[0][j] * v.x + m.r[1][j] * v.y + m.r[2][j] * v.z; }
RSG_D float cols_dot(const M3& a, int i, const M3& b, int j) {
    return a.r[0][i] * b.r[0][j] + a.r[1][i] * b.r[1][j] + a.r[2][i] * b.r[2][j];
}
// btTransformAabb(min, max, margin 0, t) (B/LinearMath/btAabbUtil2.h:166-181)
RSG_D void transform_aabb_mm(V3 mn, V3 mx, const Xf& t, V3& omn, V3& omx) {
    V3 lhe = 0.5f * (mx - mn), lc = 0.5f * (mx + mn);
    M3 ab = absolute(t.b);
    V3 c = xf_apply(t, lc);
    V3 e(dot(ab.r[0], lhe), dot(ab.r[1], lhe), dot(ab.r[2], lhe));
    omn = c - e;
    omx = c + e;
}
RSG_D void line_closest(V3 pa, V3 ua, V3 pb, V3 ub, float& alpha, float& beta) {  // dLineClosestApproach
    V3 p(pb.x - pa.x, pb.y - pa.y, pb.z - pa.z);
    float uaub = dot(ua, ub), q1 = dot(ua, p), q2 = -dot(ub, p);
    float d = 1 - uaub * uaub;
    if (d <= 0.0001f) {
        alpha = 0;
        beta = 0;
    } else {
        d = 1.f / d;
        alpha = (q1 + uaub * q2) * d;
        beta = (uaub * q1 + q2) * d;
    }
}
// intersectRectQuad2: clips quad[8] against |x| < h[0], |y| < h[1]; up to 8 points into ret
RSG_DN int clip_quad(const float h[2], const float quad[8], float ret[16]) {
    float bufA[16], bufB[16];
    for (int i = 0; i < 8; i++) bufA[i] = quad[i];
    float* q = bufA;
    float* r = ret;
    int nq = 4, nr = 0;
    bool full = false;
    for (int pass = 0; pass < 4 && !full; pass++) {
        int dir = pass >> 1;
        float sign = (pass & 1) ? 1.f : -1.f;
        float* pq = q;
        float* pr = r;
        nr = 0;
        for (int i = nq; i > 0; i--) {
            bool in = sign * pq[dir] < h[dir];
            if (in) {
                pr[0] = pq[0];
                pr[1] = pq[1];
                pr += 2;
                nr++;
                if (nr & 8) { full = true; break; }
            }
            float* nx = (i > 1) ? pq + 2 : q;
            bool nin = sign * nx[dir] < h[dir];
            if (in != nin) {
                pr[1 - dir] = pq[1 - dir] + (nx[1 - dir] - pq[1 - dir]) / (nx[dir] - pq[dir]) * (sign * h[dir] - pq[dir]);
                pr[dir] = sign * h[dir];
                pr += 2;
                nr++;
                if (nr & 8) { full = true; break; }
            }
            pq += 2;
        }
        q = r;
        if (full) break;
        r = (r == ret) ? bufB : ret;
        nq = nr;
    }
    if (q != ret)
        for (int i = 0; i < nr * 2; i++) ret[i] = q[i];
    return nr;
}
// cullPoints2: keeps m of n polygon points spread by angle around the centroid
RSG_DN void cull_points(int n, const float p[], int m, int i0, int iret[]) {
    const float PI_ODE = 3.14159265f;
    float a, cx, cy, q;
    if (n == 1) {
        cx = p[0];
        cy = p[1];
    } else if (n == 2) {
        cx = 0.5f * (p[0] + p[2]);
        cy = 0.5f * (p[1] + p[3]);
    } else {
        a = 0;
        cx = 0;
        cy = 0;
        for (int i = 0; i < n - 1; i++) {
            q = p[i * 2] * p[i * 2 + 3] - p[i * 2 + 2] * p[i * 2 + 1];
            a += q;
            cx += q * (p[i * 2] + p[i * 2 + 2]);
            cy += q * (p[i * 2 + 1] + p[i * 2 + 3]);
        }
        q = p[n * 2 - 2] * p[1] - p[0] * p[n * 2 - 1];
        if (fabsf(a + q) > SIMD_EPS) a = 1.f / (3.0f * (a + q));
        else a = BT_LARGE;
        cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
        cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
    }
    float ang[8];
    for (int i = 0; i < n; i++) ang[i] = atan2f(p[i * 2 + 1] - cy, p[i * 2] - cx);
    int avail[8];
    for (int i = 0; i < n; i++) avail[i] = 1;
    avail[i0] = 0;
    iret[0] = i0;
    for (int j = 1; j < m; j++) {
        a = (float)j * (2 * PI_ODE / m) + ang[i0];
        if (a > PI_ODE) a -= 2 * PI_ODE;
        float maxdiff = 1e9f;
        iret[j] = i0;
        for (int i = 0; i < n; i++) {
            if (avail[i]) {
                float diff = fabsf(ang[i] - a);
                if (diff > PI_ODE) diff = 2 * PI_ODE - diff;
                if (diff < maxdiff) {
                    maxdiff = diff;
                    iret[j] = i;
                }
            }
        }
        avail[iret[j]] = 0;
    }
}
// dBoxBox2 with at most 4 contacts; returns the count, `normal` is the detector's normal
RSG_DN int box_box(V3 p1, const M3& R1, V3 A, V3 p2, const M3& R2, V3 B, V3& normal, BoxHit out[4]) {
    const float fudge_factor = 1.05f;
    V3 p(p2.x - p1.x, p2.y - p1.y, p2.z - p1.z);
    float pp[3] = {col_dot(R1, 0, p), col_dot(R1, 1, p), col_dot(R1, 2, p)};
    float R[3][3], Q[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            R[i][j] = cols_dot(R1, i, R2, j);
            Q[i][j] = fabsf(R[i][j]);
        }
    float s = -FLT_MAX, s2, l;
    int normal_axis = -1, code = 0;
    V3 normalC(0.f, 0.f, 0.f);
    bool invert = false;
    float Av[3] = {A.x, A.y, A.z}, Bv[3] = {B.x, B.y, B.z};
    // face axes u1..u3 of box 1 and v1..v3 of box 2
    float fe1[6] = {pp[0], pp[1], pp[2], col_dot(R2, 0, p), col_dot(R2, 1, p), col_dot(R2, 2, p)};
    float fe2[6] = {A.x + B.x * Q[0][0] + B.y * Q[0][1] + B.z * Q[0][2], A.y + B.x * Q[1][0] + B.y * Q[1][1] + B.z * Q[1][2],
                    A.z + B.x * Q[2][0] + B.y * Q[2][1] + B.z * Q[2][2], A.x * Q[0][0] + A.y * Q[1][0] + A.z * Q[2][0] + B.x,
                    A.x * Q[0][1] + A.y * Q[1][1] + A.z * Q[2][1] + B.y, A.x * Q[0][2] + A.y * Q[1][2] + A.z * Q[2][2] + B.z};
    for (int k = 0; k < 6; k++) {
        s2 = fabsf(fe1[k]) - fe2[k];
        if (s2 > 0) return 0;
        if (s2 > s) {
            s = s2;
            normal_axis = k;
            invert = fe1[k] < 0;
            code = k + 1;
        }
    }
    const float f2 = 1.0e-5f;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Q[i][j] += f2;
    // edge axes u_i x v_j
    float ee1[9] = {pp[2] * R[1][0] - pp[1] * R[2][0], pp[2] * R[1][1] - pp[1] * R[2][1], pp[2] * R[1][2] - pp[1] * R[2][2],
                    pp[0] * R[2][0] - pp[2] * R[0][0], pp[0] * R[2][1] - pp[2] * R[0][1], pp[0] * R[2][2] - pp[2] * R[0][2],
                    pp[1] * R[0][0] - pp[0] * R[1][0], pp[1] * R[0][1] - pp[0] * R[1][1], pp[1] * R[0][2] - pp[0] * R[1][2]};
    float ee2[9] = {A.y * Q[2][0] + A.z * Q[1][0] + B.y * Q[0][2] + B.z * Q[0][1],
                    A.y * Q[2][1] + A.z * Q[1][1] + B.x * Q[0][2] + B.z * Q[0][0],
                    A.y * Q[2][2] + A.z * Q[1][2] + B.x * Q[0][1] + B.y * Q[0][0],
                    A.x * Q[2][0] + A.z * Q[0][0] + B.y * Q[1][2] + B.z * Q[1][1],
                    A.x * Q[2][1] + A.z * Q[0][1] + B.x * Q[1][2] + B.z * Q[1][0],
                    A.x * Q[2][2] + A.z * Q[0][2] + B.x * Q[1][1] + B.y * Q[1][0],
                    A.x * Q[1][0] + A.y * Q[0][0] + B.y * Q[2][2] + B.z * Q[2][1],
                    A.x * Q[1][1] + A.y * Q[0][1] + B.x * Q[2][2] + B.z * Q[2][0],
                    A.x * Q[1][2] + A.y * Q[0][2] + B.x * Q[2][1] + B.y * Q[2][0]};
    float en[9][3] = {{0, -R[2][0], R[1][0]}, {0, -R[2][1], R[1][1]}, {0, -R[2][2], R[1][2]},
                      {R[2][0], 0, -R[0][0]}, {R[2][1], 0, -R[0][1]}, {R[2][2], 0, -R[0][2]},
                      {-R[1][0], R[0][0], 0}, {-R[1][1], R[0][1], 0}, {-R[1][2], R[0][2], 0}};
    for (int k = 0; k < 9; k++) {
        s2 = fabsf(ee1[k]) - ee2[k];
        if (s2 > SIMD_EPS) return 0;
        float n1 = en[k][0], n2 = en[k][1], n3 = en[k][2];
        l = sqrtf(n1 * n1 + n2 * n2 + n3 * n3);
        if (l > SIMD_EPS) {
            s2 /= l;
            if (s2 * fudge_factor > s) {
                s = s2;
                normal_axis = -1;
                normalC = V3(n1 / l, n2 / l, n3 / l);
                invert = ee1[k] < 0;
                code = 7 + k;
            }
        }
    }
    if (!code) return 0;
    if (normal_axis >= 0) {
        const M3& Rn = normal_axis < 3 ? R1 : R2;
        int c = normal_axis % 3;
        normal = V3(Rn.r[0][c], Rn.r[1][c], Rn.r[2][c]);
    } else {
        normal = V3(dot(R1.r[0], normalC), dot(R1.r[1], normalC), dot(R1.r[2], normalC));
    }
    if (invert) normal = V3(-normal.x, -normal.y, -normal.z);
    float depth = -s;
    if (code > 6) {  // edge-edge
        V3 pb = p2;
        for (int j = 0; j < 3; j++) {
            float sign = (col_dot(R2, j, normal) > 0) ? -1.0f : 1.0f;
            for (int i = 0; i < 3; i++) pb[i] += sign * Bv[j] * R2.r[i][j];
        }
        V3 pa = p1;
        for (int j = 0; j < 3; j++) {
            float sign = (col_dot(R1, j, normal) > 0) ? 1.0f : -1.0f;
            for (int i = 0; i < 3; i++) pa[i] += sign * Av[j] * R1.r[i][j];
        }
        int ca = (code - 7) / 3, cb = (code - 7) % 3;
        V3 ua(R1.r[0][ca], R1.r[1][ca], R1.r[2][ca]), ub(R2.r[0][cb], R2.r[1][cb], R2.r[2][cb]);
        float alpha, beta;
        line_closest(pa, ua, pb, ub, alpha, beta);
        for (int i = 0; i < 3; i++) pb[i] += ub[i] * beta;
        out[0].point = pb;
        out[0].depth = depth;
        return 1;
    }
    bool a_is_1 = code <= 3;
    const M3& Ra = a_is_1 ? R1 : R2;
    const M3& Rb = a_is_1 ? R2 : R1;
    V3 pa = a_is_1 ? p1 : p2, pb = a_is_1 ? p2 : p1;
    const float* Sa = a_is_1 ? Av : Bv;
    const float* Sb = a_is_1 ? Bv : Av;
    V3 normal2 = a_is_1 ? normal : V3(-normal.x, -normal.y, -normal.z);
    float nr[3] = {col_dot(Rb, 0, normal2), col_dot(Rb, 1, normal2), col_dot(Rb, 2, normal2)};
    float anr[3] = {fabsf(nr[0]), fabsf(nr[1]), fabsf(nr[2])};
    int lanr, a1, a2;
    if (anr[1] > anr[0]) {
        if (anr[1] > anr[2]) { a1 = 0; lanr = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    } else {
        if (anr[0] > anr[2]) { lanr = 0; a1 = 1; a2 = 2; }
        else { a1 = 0; a2 = 1; lanr = 2; }
    }
    V3 center;
    for (int i = 0; i < 3; i++) {
        if (nr[lanr] < 0) center[i] = pb[i] - pa[i] + Sb[lanr] * Rb.r[i][lanr];
        else center[i] = pb[i] - pa[i] - Sb[lanr] * Rb.r[i][lanr];
    }
    int codeN = a_is_1 ? code - 1 : code - 4;
    int code1 = codeN == 0 ? 1 : 0;
    int code2 = codeN == 2 ? 1 : 2;
    float c1 = col_dot(Ra, code1, center), c2 = col_dot(Ra, code2, center);
    float m11 = cols_dot(Ra, code1, Rb, a1), m12 = cols_dot(Ra, code1, Rb, a2);
    float m21 = cols_dot(Ra, code2, Rb, a1), m22 = cols_dot(Ra, code2, Rb, a2);
    float quad[8];
    {
        float k1 = m11 * Sb[a1], k2 = m21 * Sb[a1], k3 = m12 * Sb[a2], k4 = m22 * Sb[a2];
        quad[0] = c1 - k1 - k3;
        quad[1] = c2 - k2 - k4;
        quad[2] = c1 - k1 + k3;
        quad[3] = c2 - k2 + k4;
        quad[4] = c1 + k1 + k3;
        quad[5] = c2 + k2 + k4;
        quad[6] = c1 + k1 - k3;
        quad[7] = c2 + k2 - k4;
    }
    float rect[2] = {Sa[code1], Sa[code2]};
    float ret[16];
    int n = clip_quad(rect, quad, ret);
    if (n < 1) return 0;
    float point[3 * 8], dep[8];
    float det1 = 1.f / (m11 * m22 - m12 * m21);
    m11 *= det1;
    m12 *= det1;
    m21 *= det1;
    m22 *= det1;
    int cnum = 0;
    for (int j = 0; j < n; j++) {
        float k1 = m22 * (ret[j * 2] - c1) - m12 * (ret[j * 2 + 1] - c2);
        float k2 = -m21 * (ret[j * 2] - c1) + m11 * (ret[j * 2 + 1] - c2);
        for (int i = 0; i < 3; i++) point[cnum * 3 + i] = center[i] + k1 * Rb.r[i][a1] + k2 * Rb.r[i][a2];
        dep[cnum] = Sa[codeN] - (normal2.x * point[cnum * 3] + normal2.y * point[cnum * 3 + 1] + normal2.z * point[cnum * 3 + 2]);
        if (dep[cnum] >= 0) {
            ret[cnum * 2] = ret[j * 2];
            ret[cnum * 2 + 1] = ret[j * 2 + 1];
            cnum++;
        }
    }
    if (cnum < 1) return 0;
    int maxc = cnum < 4 ? cnum : 4;
    int pick[8];
    if (cnum <= maxc) {
        for (int j = 0; j < cnum; j++) pick[j] = j;
    } else {
        int i1 = 0;
        float maxdepth = dep[0];
        for (int i = 1; i < cnum; i++)
            if (dep[i] > maxdepth) { maxdepth = dep[i]; i1 = i; }
        cull_points(cnum, ret, maxc, i1, pick);
    }
    for (int k = 0; k < maxc; k++) {
        int j = pick[k];
        V3 w(point[j * 3] + pa.x, point[j * 3 + 1] + pa.y, point[j * 3 + 2] + pa.z);
        if (code >= 4) w = w - normal * dep[j];
        out[k].point = w;
        out[k].depth = dep[j];
    }
    return maxc;
}

// ---------------------------------------------------------------- contact-added callback
RSG_D void push_event(Ctx& a, uint32_t kind, uint32_t x, uint32_t y, uint32_t flag) {
    if (!((a.event_mask >> kind) & 1u) || a.ev == nullptr) return;
    if (a.nevents >= MAX_EVENTS_PER_ARENA) {
        a.err |= ERR_EVENT_OVERFLOW;
        return;
    }
    DevEvent& e = a.ev[a.nevents++];
    e.kind = kind;
    e.tick_lo = (uint32_t)a.tick;
    e.tick_hi = (uint32_t)(a.tick >> 32);
    e.a = x;
    e.b = y;
    e.flag = flag;
}

// Arena::_BulletContactAddedCallback (src/Sim/Arena/Arena.cpp:244-414) for the point stored in
// manifold m at index idx; `tri` is the mesh triangle or -1.
RSG_DN void contact_added(const BatchView& bv, Ctx& a, Manifold& m, int idx, int tri) {
    MPoint& cp = a.pts[m.pt[idx]];
    int A = m.body0, B = m.body1;
    auto user_index = [](int o) { return o == OBJ_BALL ? 2 : (o >= OBJ_CAR0 ? 1 : -1); };
    auto responds = [&](int o) { return is_static_obj(o) ? true : !a.body(o).no_contact_response; };
    if (!responds(A) || !responds(B)) return;
    int ua = user_index(A), ub = user_index(B);
    bool swap;
    if (ua != -1 && ub != -1) swap = ua > ub;
    else swap = ub != -1;
    if (swap) {
        int t = A; A = B; B = t;
        t = ua; ua = ub; ub = t;
    }
    if (ua == 1) {
        Car& car = a.cars[A - OBJ_CAR0];
        if (ub == 2) {
            // car-ball: Ball::_OnHit (src/Sim/Ball/Ball.cpp:237-289)
            V3 rel_ball = (swap ? cp.local_a : cp.local_b) * RL::BT_TO_UU;
            V3 car_pos = car.rb.xf.o * RL::BT_TO_UU, car_vel = car.rb.lin_vel * RL::BT_TO_UU;
            V3 ball_pos = a.ball.xf.o * RL::BT_TO_UU, ball_vel = a.ball.lin_vel * RL::BT_TO_UU;
            cp.friction = RL::CARBALL_COLLISION_FRICTION;
            cp.restitution = RL::CARBALL_COLLISION_RESTITUTION;
            car.setf(F_BHI_VALID, true);
            car.bhi_rel = rel_ball;
            car.bhi_hit = a.tick;
            car.bhi_ballpos = ball_pos;
            car.bhi_extra = V3(0, 0, 0);
            push_event(a, RSG_EVENT_BALL_HIT, car.id, 0, 0);
            if ((a.tick > car.bhi_extra_tick + 1) || (car.bhi_extra_tick > a.tick)) {
                car.bhi_extra_tick = a.tick;
                V3 cf = car.fwd();
                V3 rel_pos = ball_pos - car_pos;
                V3 rel_vel = ball_vel - car_vel;
                float rs = rs_minf(rs_len(rel_vel), RL::BALL_CAR_EXTRA_IMPULSE_MAXDELTAVEL_UU);
                if (rs > 0) {
                    V3 hit = rs_normalized(rel_pos * V3(1, 1, RL::BALL_CAR_EXTRA_IMPULSE_Z_SCALE));
                    V3 adj = cf * dot(hit, cf) * (1 - RL::BALL_CAR_EXTRA_IMPULSE_FORWARD_SCALE);
                    hit = rs_normalized(hit - adj);
                    V3 added = (hit * rs) * curve_eval(c_curves[CV_BALL_EXTRA], rs) * bv.mut.ball_hit_scale;
                    car.bhi_extra = added;
                    a.ball_cache += added * RL::UU_TO_BT;
                }
                if (bv.heatseeker) {  // Ball.cpp:291-299: the touching car's team sets the target net
                    bool can_increase = (a.hs_time > RL::HS::MIN_SPEEDUP_INTERVAL) || (a.hs_dir == 0);
                    float new_dir = car.f(F_TEAM_ORANGE) ? -1.f : 1.f;
                    if (can_increase && (new_dir != a.hs_dir)) {
                        a.hs_time = 0;
                        a.hs_speed = rs_minf(a.hs_speed + RL::HS::TARGET_SPEED_INCREMENT, RL::HS::MAX_SPEED);
                    }
                    a.hs_dir = new_dir;
                }
            }
        } else if (ub == 1) {
            // car-car: Arena::_BtCallback_OnCarCarCollision (src/Sim/Arena/Arena.cpp:323-405)
            Car* c1 = &car;
            Car* c2 = &a.cars[B - OBJ_CAR0];
            cp.friction = RL::CARCAR_COLLISION_FRICTION;
            cp.restitution = RL::CARCAR_COLLISION_RESTITUTION;
            for (int i = 0; i < 2; i++) {
                bool sw = i == 1;
                if (sw) { Car* t = c1; c1 = c2; c2 = t; }
                Car& s = *c1;
                Car& o = *c2;
                if (s.f(F_DEMOED) || o.f(F_DEMOED)) return;
                if (s.cc_other == o.id && s.cc_cooldown > 0) continue;
                V3 spos = s.rb.xf.o * RL::BT_TO_UU, svel = s.rb.lin_vel * RL::BT_TO_UU;
                V3 opos = o.rb.xf.o * RL::BT_TO_UU, ovel = o.rb.lin_vel * RL::BT_TO_UU;
                V3 dp = opos - spos;
                if (dot(svel, dp) > 0) {
                    V3 vd = rs_normalized(svel);
                    V3 dir = rs_normalized(dp);
                    float sto = dot(svel, dir);
                    float oas = dot(ovel, vd);
                    if (sto > oas) {
                        V3 lp = sw ? cp.local_b : cp.local_a;
                        bool bumper = (lp.x * RL::BT_TO_UU) > RL::BUMP_MIN_FORWARD_DIST;
                        if (bumper) {
                            bool demo = bv.mut.demo_mode == 1 ? true : (bv.mut.demo_mode == 2 ? false : s.f(F_SUPERSONIC));
                            if (demo && !bv.mut.team_demos) demo = s.f(F_TEAM_ORANGE) != o.f(F_TEAM_ORANGE);
                            if (demo) {
                                o.setf(F_DEMOED, true);
                                o.demo_timer = bv.mut.respawn_delay;
                            } else {
                                bool gh = o.f(F_ON_GROUND);
                                float bs = curve_eval(c_curves[gh ? CV_BUMP_GROUND : CV_BUMP_AIR], sto);
                                V3 hu = gh ? o.up() : V3(0, 0, 1);
                                V3 bi = vd * bs + hu * curve_eval(c_curves[CV_BUMP_UP], sto) * bv.mut.bump_force_scale;
                                o.vel_cache += bi * RL::UU_TO_BT;
                            }
                            s.cc_other = o.id;
                            s.cc_cooldown = bv.mut.bump_cooldown_time;
                            push_event(a, RSG_EVENT_BUMP, s.id, o.id, demo ? 1u : 0u);
                        }
                    }
                }
            }
        } else {
            // car-world (src/Sim/Arena/Arena.cpp:407-414)
            car.setf(F_WC_CONTACT, true);
            car.wc_normal = cp.normal;
            cp.friction = bv.mut.car_world_friction;
            cp.restitution = bv.mut.car_world_restitution;
        }
    } else if (ua == 2 && ub == -1) {
        // ball-world (src/Sim/Arena/Arena.cpp:298-306): Ball::_OnWorldCollision, then special
        if (bv.heatseeker && a.hs_dir != 0) {  // Ball.cpp:326-357: a back-wall bounce turns the target around
            const V3 pos = a.ball.xf.o * RL::BT_TO_UU;
            const float rel_normal_y = cp.normal.y * a.hs_dir, rel_y = pos.y * a.hs_dir;
            if (rel_normal_y <= -RL::HS::WALL_BOUNCE_CHANGE_Y_NORMAL &&
                rel_y >= RL::ARENA_EXTENT_Y - RL::HS::WALL_BOUNCE_CHANGE_Y_THRESH) {
                a.hs_dir *= -1;
                const V3 vel = a.ball.lin_vel * RL::BT_TO_UU;
                const V3 goal(0, RL::HS::TARGET_Y * a.hs_dir, RL::HS::TARGET_Z);
                const V3 to_goal = rs_normalized(goal - pos);
                const V3 dir = to_goal * (1 - RL::HS::WALL_BOUNCE_UP_FRAC) + V3(0, 0, 1) * RL::HS::WALL_BOUNCE_UP_FRAC;
                const V3 imp = dir * rs_len(vel) * RL::HS::WALL_BOUNCE_FORCE_SCALE;
                a.ball_cache += imp * RL::UU_TO_BT;
            }
        }
        cp.special = true;
    }
#if defined(RSG_PHASE_TIMERS)
    long long ie_ = clock64();
#endif
    if (tri >= 0) adjust_internal_edge(bv.mesh, cp, tri);
#if defined(RSG_PHASE_TIMERS)
    atomicAdd(&g_phase_cycles[48], (unsigned long long)(clock64() - ie_));
#endif
}

// btManifoldResult::calculateCombined{Friction,Restitution} as RocketSim patches them
RSG_D float obj_friction(Ctx& a, int o) { return is_static_obj(o) ? RL::ARENA_COLLISION_BASE_FRICTION : a.body(o).friction; }
RSG_D float obj_restitution(Ctx& a, int o) { return is_static_obj(o) ? RL::ARENA_COLLISION_BASE_RESTITUTION : a.body(o).restitution; }
RSG_D float combined_friction(Ctx& a, int o0, int o1) {
    float x = obj_friction(a, o0), y = obj_friction(a, o1);
    if (is_static_obj(o0) || is_static_obj(o1)) return x < y ? x : y;
    return x * y;
}
RSG_D float combined_restitution(Ctx& a, int o0, int o1) {
    float x = obj_restitution(a, o0), y = obj_restitution(a, o1);
    if (is_static_obj(o0) || is_static_obj(o1)) return x > y ? x : y;
    return x * y;
}
RSG_D Xf obj_xf(Ctx& a, int o) {
    if (o < OBJ_BALL) {
        Xf t = xf_identity();
        t.o = static_origin(o);
        return t;
    }
    return a.body(o).xf;
}

// Convex object (ball sphere or car box) against the arena mesh: btConvexConcaveCollisionAlgorithm
// (B/.../CollisionDispatch/btConvexConcaveCollisionAlgorithm.cpp:71-250).  It is split in two: the
// BVH query with the per-triangle AABB and plane early-outs (which triangles reach a detector, in
// BVH order), and the detector run on one triangle.  Results are committed to the manifold in
// BVH order.
struct CandRes {
    V3 n, p;
    float d;
    int valid;
};
constexpr int MESH_SEG = 64;  // candidate triangles kept per mesh pair before falling back to lane 0
// candidate tests per round (a multiple of 32: measured 64 and 96 no faster), then lane 0 commits them
constexpr int CAND_ROUND = 32;
constexpr int HDR_LIST = 24;  // overlapping BVH subtree headers kept per mesh query

// `hdrs` (may be null) lists, in header order, the subtree headers that overlap the query box;
// without it every header is tested.
template <class F>
RSG_D void mesh_candidates(const BatchView& bv, const Xf& conv_xf, const Convex& cshape, float breaking,
                           const Subtree* subs, const int16_t* hdrs, int nh, F&& emit) {
    V3 mn, mx;
    cshape.aabb(conv_xf, mn, mx);
    M3 inv_basis = inverse(conv_xf.b);
    auto visit = [&](int t) {
        V3 tv[3];
        tri_load(bv.mesh, t, tv);
        // TestTriangleAgainstAabb2 (z, x, y)
        const int ord[3] = {2, 0, 1};
        for (int q = 0; q < 3; q++) {
            int k = ord[q];
            float lo = fminf(fminf(tv[0][k], tv[1][k]), tv[2][k]);
            float hi = fmaxf(fmaxf(tv[0][k], tv[1][k]), tv[2][k]);
            if (lo > mx[k]) return;
            if (hi < mn[k]) return;
        }
        {  // early out on the triangle plane
            V3 tn = normalized(cross(tv[1] - tv[0], tv[2] - tv[0]));
            for (int side = 0; side < 2; side++) {
                V3 dir = side ? -tn : tn;
                V3 ld = inv_basis * dir;
                V3 lp;
                if (cshape.type == 1) {
                    V3 vn = ld;
                    if (len2(vn) < SIMD_EPS * SIMD_EPS) vn = normalized(V3(-1, -1, -1));
                    else vn = normalized(vn);
                    lp = cshape.margin * vn;
                } else {
                    V3 hm = cshape.he + V3(cshape.margin, cshape.margin, cshape.margin);
                    lp = V3(ld.x >= 0 ? hm.x : -hm.x, ld.y >= 0 ? hm.y : -hm.y, ld.z >= 0 ? hm.z : -hm.z);
                }
                V3 wp = xf_apply(conv_xf, lp);
                float pp = dot(dir, wp), pt = dot(dir, tv[0]);
                if (pt - pp > breaking) return;
            }
        }
        emit(t);
    };
    if (!hdrs) {
        mesh_query_aabb(bv.mesh, mn, mx, visit);
        return;
    }
    uint16_t qa[3], qb[3];
    quantize_clamp(bv.mesh, qa, mn, false);
    quantize_clamp(bv.mesh, qb, mx, true);
    for (int i = 0; i < nh; i++) {
        uint16_t smin[3], smax[3];
        int root, size;
        subtree_load_at(subs + hdrs[i], smin, smax, root, size);
        subtree_walk(bv.mesh, qa, qb, root, size, visit);
    }
}

RSG_DN CandRes mesh_candidate_test(const BatchView& bv, const Xf& conv_xf, const Convex& cshape, float breaking, int t,
                                   uint32_t& warn) {
    V3 tv[3];
    tri_load(bv.mesh, t, tv);
    CandRes r;
    if (cshape.type == 1) {
        float depth;
        V3 point, nrm;
        r.valid = sphere_triangle(conv_xf.o, cshape.margin, tv, breaking, point, nrm, depth);
        r.n = nrm;
        r.p = point;
        r.d = depth;
    } else {
        Convex tri;
        tri.type = 2;
        tri.margin = 0.f;
        tri.he = V3(0, 0, 0);
        for (int k = 0; k < 3; k++) tri.tv[k] = tv[k];
        float md = cshape.margin + tri.margin + breaking;
        GjkOut g = gjk(cshape, conv_xf, tri, xf_identity(), md * md);
        if (g.epa_needed) warn |= WARN_EPA_SKIPPED;
        r.valid = g.valid;
        r.n = g.normal;
        r.p = g.point_on_b;
        r.d = g.dist;
    }
    return r;
}

RSG_D void commit_mesh_contact(const BatchView& bv, Ctx& a, Manifold& m, const Xf& x0, const Xf& x1, float fr, float re,
                               const CandRes& r, int t) {
    if (!r.valid) return;
    int idx = add_point(a, m, x0, x1, r.n, r.p, r.d, fr, re);
    if (idx >= 0) contact_added(bv, a, m, idx, t);
}

// Whole pair on one lane (used when a pair has more candidates than its segment holds)
RSG_DN void convex_vs_mesh(const BatchView& bv, Ctx& a, Manifold& m, int conv, const Xf& conv_xf, const Convex& cshape) {
    Xf x0 = a.body(m.body0).xf, x1 = obj_xf(a, m.body1);
    float fr = combined_friction(a, OBJ_MESH, conv), re = combined_restitution(a, OBJ_MESH, conv);
    uint32_t warn = 0;
    mesh_candidates(bv, conv_xf, cshape, m.breaking, a.sub, nullptr, 0, [&](int t) {
        CandRes r = mesh_candidate_test(bv, conv_xf, cshape, m.breaking, t, warn);
        commit_mesh_contact(bv, a, m, x0, x1, fr, re, r, t);
    });
    a.err |= warn;
    refresh(a, m, x0, x1);
}

// btConvexPlaneCollisionAlgorithm::processCollision (B/.../btConvexPlaneCollisionAlgorithm.cpp:94-161)
RSG_DN void convex_vs_plane(const BatchView& bv, Ctx& a, Manifold& m, const Xf& conv_xf, const Convex& cshape, int plane_obj) {
    PlaneC pl;
    plane_const(plane_obj - OBJ_PLANE0, pl);
    Xf pxf = xf_identity();
    pxf.o = pl.origin;
    Xf plane_in_convex = xf_mul(xf_inverse(conv_xf), pxf);
    Xf convex_in_plane = xf_mul(xf_inverse(pxf), conv_xf);
    V3 dir = plane_in_convex.b * (-pl.n);
    V3 vtx;
    if (cshape.type == 1) {
        V3 vn = dir;
        if (len2(vn) < SIMD_EPS * SIMD_EPS) vn = normalized(V3(-1, -1, -1));
        else vn = normalized(vn);
        vtx = cshape.margin * vn;
    } else {
        V3 hm = cshape.he + V3(cshape.margin, cshape.margin, cshape.margin);
        vtx = V3(dir.x >= 0 ? hm.x : -hm.x, dir.y >= 0 ? hm.y : -hm.y, dir.z >= 0 ? hm.z : -hm.z);
    }
    V3 vip = xf_apply(convex_in_plane, vtx);
    float distance = dot(pl.n, vip) - 0.f;
    Xf x0 = a.body(m.body0).xf, x1 = pxf;
    if (distance < m.breaking) {
        V3 proj = vip - distance * pl.n;
        V3 pw = xf_apply(pxf, proj);
        V3 nw = pxf.b * pl.n;
        int conv = m.body0;
        float fr = combined_friction(a, plane_obj, conv), re = combined_restitution(a, plane_obj, conv);
        int idx = add_point(a, m, x0, x1, nw, pw, distance, fr, re);
        if (idx >= 0) contact_added(bv, a, m, idx, -1);
    }
    if (m.n) refresh(a, m, x0, x1);
}

// btAlignedObjectArray::quickSortInternal (B/LinearMath/btAlignedObjectArray.h:370-400) over manifold
// indices keyed by island id; sub-ranges are disjoint, so an explicit stack gives the same result.
// stk_lo / stk_hi: scratch of at least n entries each
RSG_D void island_quicksort(const Ctx& a, int* v, int n, int* stk_lo, int* stk_hi) {
    int sp = 0;
    stk_lo[sp] = 0;
    stk_hi[sp] = n - 1;
    sp++;
    while (sp > 0) {
        sp--;
        int lo = stk_lo[sp], hi = stk_hi[sp];
        int i = lo, j = hi;
        int x = a.man[v[(lo + hi) / 2]].island;
        do {
            while (a.man[v[i]].island < x) i++;
            while (x < a.man[v[j]].island) j--;
            if (i <= j) {
                int t = v[i]; v[i] = v[j]; v[j] = t;
                i++;
                j--;
            }
        } while (i <= j);
        if (lo < j) { stk_lo[sp] = lo; stk_hi[sp] = j; sp++; }
        if (i < hi) { stk_lo[sp] = i; stk_hi[sp] = hi; sp++; }
    }
}

// ---------------------------------------------------------------- solver
// btSequentialImpulseConstraintSolver (B/BulletDynamics/ConstraintSolver/btSequentialImpulseConstraintSolver.cpp)
// in RocketSim's configuration: 10 iterations, split impulse, no warm starting (manifolds are rebuilt
// every tick), one friction direction, erp2 0.8.  A row's body B is either a dynamic body (its
// Jacobian on B is the negated normal) or the fixed body (zero); the constraint-force mixing term is
// zero for every row RocketSim builds, so rows keep neither.
constexpr int SB_FIXED = MAX_DYN;
struct SBody {
    int obj;  // -1 fixed body
    V3 dlv, dav, push, turn;
    float inv_mass;
    V3 lv, av, ext_f, ext_t;
    Xf xf;
};
struct Row {
    int8_t ba, bb, special;
    int16_t friction_index;
    V3 n1, rp1xn, rp2xn, angA, angB;
    float jac_inv, rhs, rhs_pen, applied, applied_push, friction;
};
RSG_D V3 row_n2(const Row& r) { return r.bb == SB_FIXED ? V3(0, 0, 0) : -r.n1; }

RSG_D void init_solver_body(Ctx& a, SBody& sb, int obj, float dt) {
    Body& b = a.body(obj);
    sb.obj = obj;
    sb.xf = b.xf;
    sb.inv_mass = b.inv_mass;
    sb.lv = b.lin_vel;
    sb.av = b.ang_vel;
    sb.ext_f = b.total_force * b.inv_mass * dt;
    sb.ext_t = b.total_torque * b.inv_inertia_world * dt;
    sb.dlv = sb.dav = sb.push = sb.turn = V3(0, 0, 0);
}

RSG_D void setup_contact_row(Ctx& a, Row& r, int ia, int ib, const MPoint& cp, V3 rel1, V3 rel2, float dt) {
    SBody& A = a.sb[ia];
    SBody& B = a.sb[ib];
    Body* rb0 = A.obj >= 0 ? &a.body(A.obj) : nullptr;
    Body* rb1 = B.obj >= 0 ? &a.body(B.obj) : nullptr;
    float inv_dt = 1.f / dt;
    float cfm = 0.f * inv_dt;
    const float erp = 0.8f;  // m_erp2 (src/Sim/Arena/Arena.cpp:473-475)
    r.ba = (int8_t)ia;
    r.bb = (int8_t)ib;
    V3 ta0 = cross(rel1, cp.normal);
    r.angA = rb0 ? rb0->inv_inertia_world * ta0 : V3(0, 0, 0);
    V3 ta1 = cross(rel2, cp.normal);
    r.angB = rb1 ? rb1->inv_inertia_world * (-ta1) : V3(0, 0, 0);
    float d0 = 0, d1 = 0;
    if (rb0) { V3 v = cross(r.angA, rel1); d0 = rb0->inv_mass + dot(cp.normal, v); }
    if (rb1) { V3 v = cross(-r.angB, rel2); d1 = rb1->inv_mass + dot(cp.normal, v); }
    r.jac_inv = 1.f / (d0 + d1 + cfm);
    V3 n1 = rb0 ? cp.normal : V3(0, 0, 0);
    V3 n2 = rb1 ? -cp.normal : V3(0, 0, 0);
    r.n1 = n1;
    r.rp1xn = rb0 ? ta0 : V3(0, 0, 0);
    r.rp2xn = rb1 ? -ta1 : V3(0, 0, 0);
    float restitution = 0.f;
    float penetration = cp.dist + 0.f;
    {
        V3 v1 = rb0 ? rb0->vel_at(rel1) : V3(0, 0, 0);
        V3 v2 = rb1 ? rb1->vel_at(rel2) : V3(0, 0, 0);
        float rel_vel = dot(cp.normal, v1 - v2);
        r.friction = cp.friction;
        if (fabsf(rel_vel) < 0.2f) restitution = 0.f;  // restitutionCurve, threshold 0.2
        else restitution = cp.restitution * -rel_vel;
        if (restitution <= 0.f) restitution = 0.f;
    }
    r.applied = 0.f * 0.85f;
    r.applied_push = 0.f;
    {
        V3 efA = A.obj >= 0 ? A.ext_f : V3(0, 0, 0), etA = A.obj >= 0 ? A.ext_t : V3(0, 0, 0);
        V3 efB = B.obj >= 0 ? B.ext_f : V3(0, 0, 0), etB = B.obj >= 0 ? B.ext_t : V3(0, 0, 0);
        float v1 = dot(n1, A.lv + efA) + dot(r.rp1xn, A.av + etA);
        float v2 = dot(n2, B.lv + efB) + dot(r.rp2xn, B.av + etB);
        float rel_vel = v1 + v2;
        float pos_err = 0.f;
        float vel_err = restitution - rel_vel;
        if (penetration > 0) pos_err = 0;
        else pos_err = -penetration * erp * inv_dt;
        float pen_imp = pos_err * r.jac_inv;
        float vel_imp = vel_err * r.jac_inv;
        if (penetration > 1.0e30f) {  // split impulse threshold 1e30 (src/Sim/Arena/Arena.cpp:474)
            r.rhs = pen_imp + vel_imp;
            r.rhs_pen = 0.f;
        } else {
            r.rhs = vel_imp;
            r.rhs_pen = pen_imp;
        }
    }
    r.special = cp.special;
}

RSG_D void setup_friction_row(Ctx& a, Row& r, V3 n, int ia, int ib, float friction, V3 rel1, V3 rel2) {
    SBody& A = a.sb[ia];
    SBody& B = a.sb[ib];
    Body* b0 = A.obj >= 0 ? &a.body(A.obj) : nullptr;
    Body* b1 = B.obj >= 0 ? &a.body(B.obj) : nullptr;
    r.ba = (int8_t)ia;
    r.bb = (int8_t)ib;
    r.special = 0;
    r.friction = friction;
    r.applied = 0;
    r.applied_push = 0;
    V3 n1 = b0 ? n : V3(0, 0, 0), n2 = b1 ? -n : V3(0, 0, 0);
    r.n1 = n1;
    if (b0) {
        V3 t = cross(rel1, n1);
        r.rp1xn = t;
        r.angA = b0->inv_inertia_world * t;
    } else {
        r.rp1xn = r.angA = V3(0, 0, 0);
    }
    if (b1) {
        V3 t = cross(rel2, n2);
        r.rp2xn = t;
        r.angB = b1->inv_inertia_world * t;
    } else {
        r.rp2xn = r.angB = V3(0, 0, 0);
    }
    float d0 = 0, d1 = 0;
    if (b0) { V3 v = cross(r.angA, rel1); d0 = b0->inv_mass + dot(n, v); }
    if (b1) { V3 v = cross(-r.angB, rel2); d1 = b1->inv_mass + dot(n, v); }
    r.jac_inv = 1.f / (d0 + d1);
    float v1 = dot(n1, b0 ? A.lv + A.ext_f : V3(0, 0, 0)) + dot(r.rp1xn, b0 ? A.av : V3(0, 0, 0));
    float v2 = dot(n2, b1 ? B.lv + B.ext_f : V3(0, 0, 0)) + dot(r.rp2xn, b1 ? B.av : V3(0, 0, 0));
    float rel_vel = v1 + v2;
    float vel_imp = (0.f - rel_vel) * r.jac_inv;
    r.rhs = 0.f + vel_imp;
    r.rhs_pen = 0.f;
}

// convertContactInner friction part (btSequentialImpulseConstraintSolver.cpp:1071-1162)
RSG_D void add_friction(Ctx& a, int& nf, int ia, int ib, V3 normal, float friction, V3 rel1, V3 rel2, int fidx) {
    SBody& A = a.sb[ia];
    SBody& B = a.sb[ib];
    V3 v1 = A.obj >= 0 ? A.lv + A.ext_f + cross(A.av + A.ext_t, rel1) : V3(0, 0, 0);
    V3 v2 = B.obj >= 0 ? B.lv + B.ext_f + cross(B.av + B.ext_t, rel2) : V3(0, 0, 0);
    V3 vel = v1 - v2;
    float rel_vel = dot(normal, vel);
    V3 lat = vel - normal * rel_vel;
    float lat2 = len2(lat);
    V3 dir;
    if (lat2 > SIMD_EPS) {
        dir = lat * (1.f / sqrtf(lat2));
    } else {
        V3 d2;
        plane_space(normal, dir, d2);
    }
    Row& fr = a.rows_f[nf++];
    fr.friction_index = (int16_t)fidx;
    setup_friction_row(a, fr, dir, ia, ib, friction, rel1, rel2);
}

// gResolveSingleConstraintRowGeneric / LowerLimit with the row's limits passed in
RSG_D void solve_row(Ctx& a, Row& c, float lo, float hi, bool lower_only) {
    SBody& A = a.sb[c.ba];
    SBody& B = a.sb[c.bb];
    V3 n2 = row_n2(c);
    float d = c.rhs - c.applied * 0.f;
    float d1 = simd_dot(c.n1, A.dlv) + simd_dot(c.rp1xn, A.dav);
    float d2 = simd_dot(n2, B.dlv) + simd_dot(c.rp2xn, B.dav);
    d -= d1 * c.jac_inv;
    d -= d2 * c.jac_inv;
    float sum = c.applied + d;
    if (sum < lo) { d = lo - c.applied; c.applied = lo; }
    else if (!lower_only && sum > hi) { d = hi - c.applied; c.applied = hi; }
    else c.applied = sum;
    if (A.obj >= 0) { A.dlv += c.n1 * A.inv_mass * d; A.dav += c.angA * d; }
    if (B.obj >= 0) { B.dlv += n2 * B.inv_mass * d; B.dav += c.angB * d; }
}

// Whether the squared split-impulse residual the reference returns, (float)(d * (1. / jac_inv)) computed
// in double and squared in float, is positive: all the split iterations use it for (their stop test
// compares the largest square with 0).  Clear cases are decided in float (the double value agrees
// with |d| / |jac_inv| to a few float ulps, so it squares to at least 2^-120 above 2^-60 and rounds
// to 0 below 2^-90); the band between, NaN and infinity take the reference's double arithmetic.
RSG_D bool split_residual_positive(float d, float jac_inv) {
    if (d == 0.f) return false;
    const float q = fabsf(d) / fabsf(jac_inv);
    if (q > 8.673617e-19f) return true;   // 2^-60
    if (q < 8.077936e-28f) return false;  // 2^-90
    const float res = (float)((double)d * (1. / (double)jac_inv));
    return res * res > 0.f;
}

// gResolveSplitPenetrationImpulse_sse2; returns split_residual_positive of its impulse change
RSG_D bool solve_split(Ctx& a, Row& c) {
    if (!c.rhs_pen) return false;
    SBody& A = a.sb[c.ba];
    SBody& B = a.sb[c.bb];
    V3 n2 = row_n2(c);
    float d = c.rhs_pen - c.applied_push * 0.f;
    float d1 = simd_dot(c.n1, A.push) + simd_dot(c.rp1xn, A.turn);
    float d2 = simd_dot(n2, B.push) + simd_dot(c.rp2xn, B.turn);
    d -= d1 * c.jac_inv;
    d -= d2 * c.jac_inv;
    float sum = c.applied_push + d;
    if (sum < 0.f) { d = 0.f - c.applied_push; c.applied_push = 0.f; }
    else c.applied_push = sum;
    if (A.obj >= 0) { A.push += c.n1 * A.inv_mass * d; A.turn += c.angA * d; }
    if (B.obj >= 0) { B.push += n2 * B.inv_mass * d; B.turn += c.angB * d; }
    return split_residual_positive(d, c.jac_inv);
}

// The solver (btSequentialImpulseConstraintSolver::solveGroup) in three parts: solve_plan (lane 0)
// fixes the solver bodies and the contact rows in Bullet's order and adds up RocketSim's special
// contacts per body; solve_setup_warp sets the rows up on the warp's lanes (each row reads only its
// contact point and the solver bodies' start state); solve_iterate_warp runs the iterations, a lane
// per component of solver bodies joined by rows, and writes the bodies back.  `bodies` are dynamic object ids in island order, `mans` manifold indices in
// sorted island order, `plan` room for one word per row.
RSG_DN void solve_plan(Ctx& a, const int* bodies, int nb, const int* mans, int nm, int* plan) {
    int nc = 0;
    for (int i = 0; i < MAX_DYN; i++) a.sb_of[i] = -1;
    for (int i = 0; i < nb; i++) a.sb_of[bodies[i] - OBJ_BALL] = (int8_t)i;
    auto sbi = [&](int o) { return is_static_obj(o) ? SB_FIXED : (int)a.sb_of[o - OBJ_BALL]; };
    for (int mi = 0; mi < nm; mi++) {
        Manifold& m = a.man[mans[mi]];
        int ia = sbi(m.body0), ib = sbi(m.body1);
        if (ia < 0 || ib < 0) continue;
        for (int j = 0; j < m.n; j++) {
            const MPoint& cp = a.pts[m.pt[j]];
            if (!(cp.dist <= BT_LARGE)) continue;
            if (nc >= a.cap_rows) { a.err |= ERR_ROW_OVERFLOW; continue; }
            plan[nc++] = (mans[mi] << 2) | j;
            if (cp.special) {  // the special contact sums, in row order (convertContactSpecial's inputs)
                V3 rel1 = cp.pos_a - obj_xf(a, m.body0).o;
                V3 rel2 = cp.pos_b - obj_xf(a, m.body1).o;
                for (int k = 0; k < 2; k++) {
                    int o = k ? m.body1 : m.body0;
                    if (!is_static_obj(o)) {
                        Body& b = a.body(o);
                        b.n_special++;
                        b.sp_friction = cp.friction;
                        b.sp_restitution = cp.restitution;
                        b.sp_total_normal += cp.normal;
                        b.sp_total_dist += len(k ? rel2 : rel1);
                    }
                }
            }
        }
    }
    // RocketSim's averaged ball-world contact (convertContactSpecial,
    // btSequentialImpulseConstraintSolver.cpp:1164-1211): one row per body with special contacts,
    // in body order after the others
    int nsp = 0;
    for (int i = 0; i < nb; i++) {
        Body& b = a.body(bodies[i]);
        if (b.n_special > 0) {
            if (nc + nsp < a.cap_rows) {
                a.solve_special[nsp++] = (int8_t)i;
            } else {
                a.err |= ERR_ROW_OVERFLOW;
                b.n_special = 0;
                b.sp_friction = b.sp_restitution = b.sp_total_dist = 0;
                b.sp_total_normal = V3(0, 0, 0);
            }
        }
    }
    a.solve_bodies = const_cast<int*>(bodies);
    a.solve_plan = plan;
    a.solve_nb = nb;
    a.solve_nc = nc;
    a.solve_nsp = nsp;
}

RSG_D void solve_setup_warp(Ctx& a, int lane, float dt) {
    const int nb = a.solve_nb, nc = a.solve_nc, nsp = a.solve_nsp;
    if (lane < nb) init_solver_body(a, a.sb[lane], a.solve_bodies[lane], dt);
    if (lane == 31) {
        SBody& fixed = a.sb[SB_FIXED];
        fixed.obj = -1;
        fixed.xf = xf_identity();
        fixed.inv_mass = 0;
        fixed.dlv = fixed.dav = fixed.push = fixed.turn = fixed.lv = fixed.av = fixed.ext_f = fixed.ext_t = V3(0, 0, 0);
    }
    __syncwarp();
    auto sbi = [&](int o) { return is_static_obj(o) ? SB_FIXED : (int)a.sb_of[o - OBJ_BALL]; };
    for (int k = lane; k < nc; k += 32) {
        const int e = a.solve_plan[k];
        const Manifold& m = a.man[e >> 2];
        const MPoint& cp = a.pts[m.pt[e & 3]];
        const int ia = sbi(m.body0), ib = sbi(m.body1);
        Row& r = a.rows_c[k];
        V3 rel1 = cp.pos_a - obj_xf(a, m.body0).o;
        V3 rel2 = cp.pos_b - obj_xf(a, m.body1).o;
        setup_contact_row(a, r, ia, ib, cp, rel1, rel2, dt);
        r.friction_index = (int16_t)k;
        int nf = k;
        add_friction(a, nf, ia, ib, cp.normal, cp.friction, rel1, rel2, k);
    }
    for (int q = lane; q < nsp; q += 32) {
        const int i = a.solve_special[q], k = nc + q;
        Body& b = a.body(a.solve_bodies[i]);
        float dist = b.sp_total_dist / b.n_special;
        V3 nrm = b.sp_total_normal / (float)b.n_special;
        MPoint tmp;
        tmp.dist = dist;
        tmp.normal = nrm;
        tmp.friction = b.sp_friction;
        tmp.restitution = b.sp_restitution;
        tmp.special = false;
        Row& r = a.rows_c[k];
        V3 rel1 = nrm * -dist, rel2(0, 0, 0);
        setup_contact_row(a, r, i, SB_FIXED, tmp, rel1, rel2, dt);
        r.friction_index = (int16_t)k;
        int nf = k;
        add_friction(a, nf, i, SB_FIXED, tmp.normal, tmp.friction, rel1, rel2, k);
        b.n_special = 0;
        b.sp_friction = b.sp_restitution = b.sp_total_dist = 0;
        b.sp_total_normal = V3(0, 0, 0);
    }
}

// Solver bodies joined by a row form a component; rows of different components touch different bodies
// (the fixed body takes no impulse), so each component's rows can run on their own lane, in their order,
// and every body sees the same operations as in the reference's single pass over all rows.  Lane 0
// lists the rows by component (a stable counting sort: contact rows, then friction rows).
RSG_DN void solve_components(Ctx& a) {
    const int nb = a.solve_nb, nc = a.solve_nc + a.solve_nsp, nf = nc;
    int par[MAX_DYN + 1], cid[MAX_DYN + 1];
    for (int i = 0; i <= MAX_DYN; i++) { par[i] = i; cid[i] = -1; }
    auto find = [&](int x) {
        while (par[x] != x) x = par[x];
        return x;
    };
    for (int k = 0; k < nc; k++) {
        const Row& r = a.rows_c[k];
        if (r.ba != SB_FIXED && r.bb != SB_FIXED) {
            const int x = find(r.ba), y = find(r.bb);
            if (x != y) par[x > y ? x : y] = x < y ? x : y;
        }
    }
    int ncomp = 0;
    auto comp = [&](const Row& r) {
        const int root = find(r.ba != SB_FIXED ? r.ba : r.bb);
        if (cid[root] < 0) cid[root] = ncomp++;
        return cid[root];
    };
    int16_t* pc = a.solve_perm;
    int16_t* pf = pc + a.cap_rows;
    int16_t* sc = pf + a.cap_rows;
    int16_t* sf = sc + (MAX_DYN + 2);
    for (int i = 0; i < MAX_DYN + 2; i++) sc[i] = sf[i] = 0;
    for (int k = 0; k < nc; k++) sc[comp(a.rows_c[k]) + 1]++;
    for (int k = 0; k < nf; k++) sf[comp(a.rows_f[k]) + 1]++;
    for (int i = 0; i < ncomp; i++) { sc[i + 1] += sc[i]; sf[i + 1] += sf[i]; }
    int16_t fc[MAX_DYN + 1], ff[MAX_DYN + 1];
    for (int i = 0; i < ncomp; i++) { fc[i] = sc[i]; ff[i] = sf[i]; }
    for (int k = 0; k < nc; k++) pc[fc[comp(a.rows_c[k])]++] = (int16_t)k;
    for (int k = 0; k < nf; k++) pf[ff[comp(a.rows_f[k])]++] = (int16_t)k;
    a.solve_ncomp = ncomp;
}

// The split-impulse and the ten solver iterations with a lane per component (the split iterations'
// stop test is one vote of the warp: whether any row's residual is positive), then the bodies written
// back, a lane per body.
RSG_D void solve_iterate_warp(Ctx& a, int lane, float dt) {
    if (lane == 0) solve_components(a);
    __syncwarp();
    const int nb = a.solve_nb, ncomp = a.solve_ncomp;
    const int16_t* pc = a.solve_perm;
    const int16_t* pf = pc + a.cap_rows;
    const int16_t* sc = pf + a.cap_rows;
    const int16_t* sf = sc + (MAX_DYN + 2);
    const int ITER = 10;
    const bool mine = lane < ncomp;
    const int c0 = mine ? sc[lane] : 0, c1 = mine ? sc[lane + 1] : 0;
    const int f0 = mine ? sf[lane] : 0, f1 = mine ? sf[lane + 1] : 0;
    for (int it = 0; it < ITER; it++) {
        bool any = false;
        for (int j = c0; j < c1; j++) any |= solve_split(a, a.rows_c[pc[j]]);
        if (!__any_sync(0xffffffffu, any) || it >= ITER - 1) break;
    }
    for (int it = 0; it < ITER; it++) {
        for (int j = c0; j < c1; j++) {
            Row& r = a.rows_c[pc[j]];
            if (r.special) continue;
            solve_row(a, r, 0.f, 1e10f, true);
        }
        for (int j = f0; j < f1; j++) {
            Row& f = a.rows_f[pf[j]];
            float total = a.rows_c[f.friction_index].applied;
            if (total > 0.f) solve_row(a, f, -(f.friction * total), f.friction * total, false);
        }
    }
    __syncwarp();
    // writeBackBodies (btSequentialImpulseConstraintSolver.cpp:1878-1904)
    for (int i = lane; i < nb; i += 32) {
        SBody& sb = a.sb[i];
        Body& b = a.body(sb.obj);
        sb.lv += sb.dlv;
        sb.av += sb.dav;
        if (sb.push.x != 0.f || sb.push.y != 0 || sb.push.z != 0 || sb.turn.x != 0.f || sb.turn.y != 0 || sb.turn.z != 0) {
            Xf nt;
            integrate_transform(sb.xf, sb.push, sb.turn * 0.1f, dt, b.no_rot, nt);
            sb.xf = nt;
        }
        b.lin_vel = sb.lv + sb.ext_f;
        b.ang_vel = sb.av + sb.ext_t;
        b.xf = sb.xf;
    }
    __syncwarp();
}

// ---------------------------------------------------------------- world step
// btDiscreteDynamicsWorld::stepSimulation with one fixed substep as RocketSim drives it
// (src/Sim/Arena/Arena.cpp:731, B/BulletDynamics/Dynamics/btDiscreteDynamicsWorld.cpp:360-450)
RSG_D uint32_t grid_cell_index(const DevGrid& g, int i, int j, int k) { return (uint32_t)(i * g.ny * g.nz + j * g.nz + k); }

RSG_D bool has_pair(const Ctx& a, int x, int y) {
    for (int p = 0; p < a.npairs; p++)
        if ((a.pair0[p] == x && a.pair1[p] == y) || (a.pair0[p] == y && a.pair1[p] == x)) return true;
    return false;
}
RSG_D void add_pair(Ctx& a, int x, int y) {
    if (a.npairs >= a.cap_pairs) { a.err |= ERR_PAIR_OVERFLOW; return; }
    a.pair0[a.npairs] = (int8_t)x;
    a.pair1[a.npairs] = (int8_t)y;
    a.npairs++;
}
RSG_D Manifold& new_manifold(Ctx& a, int b0, int b1, float breaking) {
    Manifold& m = a.man[a.nman++];
    m.body0 = (int8_t)b0;
    m.body1 = (int8_t)b1;
    m.n = 0;
    m.island = -1;
    m.breaking = breaking;
    return m;
}

// Phase 1 of a world step, one lane per dynamic object (ball = lane 0, cars = lanes 1..): gravity,
// damping and predicted transform, broadphase AABB and voxel cell.  Cell changes take their sequence
// numbers in object order (a ballot prefix count), like the reference's serial AABB update.
// Angle::FromVec (src/Math/MathTypes/MathTypes.cpp:80-100): yaw and pitch of a direction
RSG_D void angle_from_vec(V3 f, float& yaw, float& pitch) {
    if (fabsf(f.y) > FLT_EPSILON || fabsf(f.x) > FLT_EPSILON) {
        yaw = atan2f(f.y, f.x);
        float dist2d = sqrtf(f.x * f.x + f.y * f.y);
        pitch = -atan2f(-f.z, dist2d);
    } else {
        yaw = 0;
        if (f.z > FLT_EPSILON) pitch = (float)(3.14159265358979323846 / 2);
        else if (f.z < -FLT_EPSILON) pitch = (float)(-3.14159265358979323846 / 2);
        else pitch = 0;
    }
}
// Math::WrapNormalizeFloat (src/Math/Math.cpp:66-73)
RSG_D float wrap_normalize(float val, float minmax) {
    float r = fmodf(val, minmax * 2);
    if (r > minmax) r -= minmax * 2;
    else if (r < -minmax) r += minmax * 2;
    return r;
}
// Math::RoundAngleUE3 (src/Math/Math.cpp:75-91): to UE3 rotator units, the low two bits dropped
RSG_D float round_angle_ue3(float ang) {
    const float TO_INTS = (float)((float)(1 << 15) / 3.14159265358979323846);
    const float BACK_TO_RADIANS = (1.f / TO_INTS) * 4.f;
    int r = ((int)(ang * TO_INTS) >> 2) & (0x4000 - 1);
    return r * BACK_TO_RADIANS;
}

// Ball::_PreTickUpdate for heatseeker (src/Sim/Ball/Ball.cpp:161-207): once a touch has given the
// ball a target net, it turns towards it and blends its speed towards the target speed.
RSG_D void ball_pre_tick_heatseeker(const BatchView& bv, Ctx& a) {
    if (a.hs_dir == 0) return;
    Body& b = a.ball;
    const V3 pos = b.xf.o * RL::BT_TO_UU, vel = b.lin_vel * RL::BT_TO_UU;
    float vyaw, vpitch, gyaw, gpitch;
    angle_from_vec(vel, vyaw, vpitch);
    const V3 goal(0, RL::HS::TARGET_Y * a.hs_dir, RL::HS::TARGET_Z);
    angle_from_vec(goal - pos, gyaw, gpitch);
    // Angle::operator- is GetDeltaTo, which wraps the delta too (MathTypes.h:306-320)
    const float dyaw = wrap_normalize(gyaw - vyaw, (float)3.14159265358979323846);
    const float dpitch = wrap_normalize(gpitch - vpitch, (float)(3.14159265358979323846 / 2));
    const float cur_speed = rs_len(vel);
    const float speed_ratio = cur_speed / RL::HS::MAX_SPEED;
    const float base = speed_ratio * bv.dt;
    float yaw = vyaw + dyaw * base * RL::HS::HORIZONTAL_BLEND;
    float pitch = vpitch + dpitch * base * RL::HS::VERTICAL_BLEND;
    yaw = wrap_normalize(yaw, (float)3.14159265358979323846);  // Angle::NormalizeFix
    pitch = wrap_normalize(pitch, (float)(3.14159265358979323846 / 2));
    pitch = rs_clampf(pitch, -RL::HS::MAX_TURN_PITCH, RL::HS::MAX_TURN_PITCH);
    yaw = round_angle_ue3(yaw);
    pitch = round_angle_ue3(pitch);
    const float new_speed = cur_speed + ((a.hs_speed - cur_speed) * RL::HS::SPEED_BLEND);
    // Angle::GetForwardVec (MathTypes.cpp:102-110)
    const float cp = cosf(-pitch), cy = cosf(yaw), sy = sinf(yaw), sp = sinf(-pitch);
    const V3 dir(cp * cy, cp * sy, -sp);
    b.lin_vel = (dir * new_speed) * RL::UU_TO_BT;
    a.hs_time += bv.dt;
}

RSG_D void step_bodies_pre(const BatchView& bv, Ctx& a, int lane) {
    const float dt = bv.dt;
    const int nd = 1 + a.ncars;
    if (bv.heatseeker) {  // Ball::_PreTickUpdate runs after the cars' and pads' (Arena.cpp:705-716)
        if (lane == 0) ball_pre_tick_heatseeker(bv, a);
        __syncwarp();
    }
    bool changed = false;
    if (lane < nd) {
        Body& b = a.body(OBJ_BALL + lane);
        // applyGravity (btDiscreteDynamicsWorld.cpp:265-277)
        if (b.is_active()) b.total_force += V3(bv.mut.grav_bt[0], bv.mut.grav_bt[1], bv.mut.grav_bt[2]) * (1.f / b.inv_mass);
        // predictUnconstraintMotion (btDiscreteDynamicsWorld.cpp:1029-1044)
        b.lin_vel *= powf(1.f - b.lin_damping, dt);
        b.ang_vel *= powf(1.f - 0.f, dt);
        integrate_transform(b.xf, b.lin_vel, b.ang_vel, dt, b.no_rot, b.interp);
        // updateSingleAabb + btRSBroadphase::setAabb
        V3 mn, mx, mn2, mx2;
        if (lane == 0) {
            ball_aabb(b.xf, a.ball_r, mn, mx);
            ball_aabb(b.interp, a.ball_r, mn2, mx2);
        } else {
            Car& c = a.cars[lane - 1];
            car_compound_aabb(c, b.xf, mn, mx);
            car_compound_aabb(c, b.interp, mn2, mx2);
        }
        V3 th(0.02f, 0.02f, 0.02f);
        mn -= th; mx += th;
        mn2 -= th; mx2 += th;
        mn = vmin(mn, mn2);
        mx = vmax(mx, mx2);
        b.bp_min = mn;
        b.bp_max = mx;
        int i, j, k;
        grid_idx(bv.grid, mn, i, j, k);
        uint32_t nidx = grid_cell_index(bv.grid, i, j, k);
        if (b.cell != nidx) {
            changed = true;
            b.cell = nidx;
            b.ci = i; b.cj = j; b.ck = k;
        }
    }
    unsigned mask = __ballot_sync(0xffffffffu, changed);
    if (changed) a.body(OBJ_BALL + lane).cell_seq = a.seq + __popc(mask & ((1u << lane) - 1u));
    __syncwarp();
    if (lane == 0) a.seq += __popc(mask);
    __syncwarp();
}

// Phase 2 of a world step: broadphase pairs (lane 0), narrow phase (candidate tests on all
// lanes, results committed in pair order by lane 0), islands and the solver (lane 0).
enum PairKind : int8_t { PK_SKIP = 0, PK_BALL_MESH, PK_BALL_PLANE, PK_CAR_MESH, PK_CAR_PLANE, PK_CAR_BALL, PK_CAR_CAR };


// calculateOverlappingPairs (btRSBroadphase.cpp:392-468) and the dispatcher's choice of algorithm
RSG_DN void build_pairs(const BatchView& bv, Ctx& a) {
    const int nd = 1 + a.ncars;
    a.npairs = 0;
    V3 mesh_mn, mesh_mx;
    if (bv.has_arena) {
        mesh_aabb(bv.mesh, mesh_mn, mesh_mx);
        mesh_mn -= V3(0.02f, 0.02f, 0.02f);
        mesh_mx += V3(0.02f, 0.02f, 0.02f);
    }
    for (int d = 0; d < nd; d++) {
        int o = OBJ_BALL + d;
        Body& b = a.body(o);
        if (bv.has_arena) {
            if (bv.mesh.cells[b.cell] && aabb_overlap(b.bp_min, b.bp_max, mesh_mn, mesh_mx))
                if (!has_pair(a, OBJ_MESH, o)) add_pair(a, OBJ_MESH, o);
            for (int p = 0; p < 4; p++) {
                PlaneC pl;
                plane_const(p, pl);
                if (aabb_overlap(b.bp_min, b.bp_max, pl.bp_min, pl.bp_max))
                    if (!has_pair(a, OBJ_PLANE0 + p, o)) add_pair(a, OBJ_PLANE0 + p, o);
            }
        }
        int cd[MAX_CARS + 1];
        int ncd = cell_dyn_list(a, b.ci, b.cj, b.ck, cd);
        if (ncd > 1) {
            for (int qi = 0; qi < ncd; qi++) {
                int q = cd[qi];
                if (q == o) continue;
                Body& bq = a.body(q);
                if (aabb_overlap(b.bp_min, b.bp_max, bq.bp_min, bq.bp_max) && !has_pair(a, o, q))
                    add_pair(a, o < q ? o : q, o < q ? q : o);
            }
        }
    }
    for (int pi = 0; pi < a.npairs; pi++) {
        int o0 = a.pair0[pi], o1 = a.pair1[pi];
        int8_t k = PK_SKIP;
        bool act0 = is_static_obj(o0) ? false : a.body(o0).is_active();
        bool act1 = a.body(o1).is_active();
        if (act0 || act1) {  // btCollisionDispatcher::needsCollision
            if (is_static_obj(o0)) {
                if (o1 == OBJ_BALL) {
                    k = o0 == OBJ_MESH ? PK_BALL_MESH : PK_BALL_PLANE;
                } else {
                    Car& c = a.cars[o1 - OBJ_CAR0];
                    Xf cx;
                    car_child_xf(c, cx);
                    V3 bmn, bmx, omn, omx;
                    car_box_aabb(c, cx, bmn, bmx);
                    if (o0 == OBJ_MESH) mesh_aabb(bv.mesh, omn, omx);
                    else {
                        PlaneC pl;
                        plane_const(o0 - OBJ_PLANE0, pl);
                        omn = pl.raw_min;
                        omx = pl.raw_max;
                    }
                    if (aabb_overlap(bmn, bmx, omn, omx)) k = o0 == OBJ_MESH ? PK_CAR_MESH : PK_CAR_PLANE;
                }
            } else if (o0 == OBJ_BALL) {
                Car& c = a.cars[o1 - OBJ_CAR0];
                Xf cx;
                car_child_xf(c, cx);
                V3 bmn, bmx, smn, smx;
                car_box_aabb(c, cx, bmn, bmx);
                ball_aabb(a.ball.xf, a.ball_r, smn, smx);
                if (aabb_overlap(bmn, bmx, smn, smx)) k = PK_CAR_BALL;
            } else {
                k = PK_CAR_CAR;
            }
        }
        a.pkind[pi] = k;
    }
}

// build_pairs spread over the warp, one lane per dynamic object: each lane lists its object's
// pairs in the order the serial loop adds them, drops the dynamic pairs that an earlier object
// already added (the serial loop's has_pair), and the lists are concatenated in object order.
RSG_D int8_t classify_pair(const BatchView& bv, Ctx& a, int o0, int o1) {
    int8_t k = PK_SKIP;
    bool act0 = is_static_obj(o0) ? false : a.body(o0).is_active();
    bool act1 = a.body(o1).is_active();
    if (act0 || act1) {  // btCollisionDispatcher::needsCollision
        if (is_static_obj(o0)) {
            if (o1 == OBJ_BALL) {
                k = o0 == OBJ_MESH ? PK_BALL_MESH : PK_BALL_PLANE;
            } else {
                Car& c = a.cars[o1 - OBJ_CAR0];
                Xf cx;
                car_child_xf(c, cx);
                V3 bmn, bmx, omn, omx;
                car_box_aabb(c, cx, bmn, bmx);
                if (o0 == OBJ_MESH) mesh_aabb(bv.mesh, omn, omx);
                else {
                    PlaneC pl;
                    plane_const(o0 - OBJ_PLANE0, pl);
                    omn = pl.raw_min;
                    omx = pl.raw_max;
                }
                if (aabb_overlap(bmn, bmx, omn, omx)) k = o0 == OBJ_MESH ? PK_CAR_MESH : PK_CAR_PLANE;
            }
        } else if (o0 == OBJ_BALL) {
            Car& c = a.cars[o1 - OBJ_CAR0];
            Xf cx;
            car_child_xf(c, cx);
            V3 bmn, bmx, smn, smx;
            car_box_aabb(c, cx, bmn, bmx);
            ball_aabb(a.ball.xf, a.ball_r, smn, smx);
            if (aabb_overlap(bmn, bmx, smn, smx)) k = PK_CAR_BALL;
        } else {
            k = PK_CAR_CAR;
        }
    }
    return k;
}
RSG_D void build_pairs_warp(const BatchView& bv, Ctx& a, int lane) {
    const int nd = 1 + a.ncars;
    constexpr int LMAX = 5 + MAX_DYN;
    int8_t l0[LMAX], l1[LMAX];
    int n = 0, ncd = 0;
    int cd[MAX_CARS + 1];
    const int o = OBJ_BALL + lane;
    if (lane < nd) ncd = cell_dyn_list(a, a.body(o).ci, a.body(o).cj, a.body(o).ck, cd);
    if (lane < nd) {
        Body& b = a.body(o);
        if (bv.has_arena) {
            V3 mesh_mn, mesh_mx;
            mesh_aabb(bv.mesh, mesh_mn, mesh_mx);
            mesh_mn -= V3(0.02f, 0.02f, 0.02f);
            mesh_mx += V3(0.02f, 0.02f, 0.02f);
            if (bv.mesh.cells[b.cell] && aabb_overlap(b.bp_min, b.bp_max, mesh_mn, mesh_mx)) {
                l0[n] = OBJ_MESH; l1[n] = (int8_t)o; n++;
            }
            for (int p = 0; p < 4; p++) {
                PlaneC pl;
                plane_const(p, pl);
                if (aabb_overlap(b.bp_min, b.bp_max, pl.bp_min, pl.bp_max)) {
                    l0[n] = (int8_t)(OBJ_PLANE0 + p); l1[n] = (int8_t)o; n++;
                }
            }
        }
    }
    int ncd_lane[MAX_DYN];
    for (int d = 0; d < MAX_DYN; d++) ncd_lane[d] = __shfl_sync(0xffffffffu, ncd, d);
    if (lane < nd && ncd > 1) {
        Body& b = a.body(o);
        for (int qi = 0; qi < ncd; qi++) {
            int q = cd[qi];
            if (q == o) continue;
            Body& bq = a.body(q);
            if (!aabb_overlap(b.bp_min, b.bp_max, bq.bp_min, bq.bp_max)) continue;
            // added already while the earlier object q listed its own pairs?
            bool earlier = q < o && ncd_lane[q - OBJ_BALL] > 1 && dyn_registered(b, bq.ci, bq.cj, bq.ck);
            if (earlier) continue;
            l0[n] = (int8_t)(o < q ? o : q);
            l1[n] = (int8_t)(o < q ? q : o);
            n++;
        }
    }
    // concatenate in object order
    int off = n;
    for (int d = 1; d < 32; d <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, off, d);
        if (lane >= d) off += v;
    }
    const int total = __shfl_sync(0xffffffffu, off, 31);
    off -= n;
    for (int i = 0; i < n; i++) {
        int at = off + i;
        if (at >= a.cap_pairs) break;
        a.pair0[at] = l0[i];
        a.pair1[at] = l1[i];
        a.pkind[at] = classify_pair(bv, a, l0[i], l1[i]);
    }
    __syncwarp();
    if (lane == 0) {
        a.npairs = total < a.cap_pairs ? total : a.cap_pairs;
        if (total > a.cap_pairs) a.err |= ERR_PAIR_OVERFLOW;
    }
    __syncwarp();
}

// collision shape of a dynamic object against static geometry
RSG_D void dyn_shape(Ctx& a, int o, Xf& xf, Convex& sh, float& breaking) {
    sh.he = V3(0, 0, 0);
    if (o == OBJ_BALL) {
        xf = a.ball.xf;
        sh.type = 1;
        sh.margin = a.ball_r;
        breaking = a.ball_breaking;
    } else {
        Car& c = a.cars[o - OBJ_CAR0];
        car_child_xf(c, xf);
        sh.type = 0;
        sh.he = car_he(c);
        sh.margin = c.cfg->margin;
        breaking = c.cfg->breaking;
    }
}

// the car-ball detector: GJK between the car's box child and the ball sphere
RSG_D CandRes car_ball_test(Ctx& a, int car_obj, uint32_t& warn) {
    Car& c = a.cars[car_obj - OBJ_CAR0];
    Xf cx;
    car_child_xf(c, cx);
    Convex box;
    box.type = 0;
    box.he = car_he(c);
    box.margin = c.cfg->margin;
    Convex sph;
    sph.type = 1;
    sph.margin = a.ball_r;
    sph.he = V3(0, 0, 0);
    float br = c.cfg->breaking < a.ball_breaking ? c.cfg->breaking : a.ball_breaking;
    float md = box.margin + sph.margin + br;
    GjkOut g = gjk(box, cx, sph, a.ball.xf, md * md);
    if (g.epa_needed) warn |= WARN_EPA_SKIPPED;
    CandRes r;
    r.valid = g.valid;
    r.n = g.normal;
    r.p = g.point_on_b;
    r.d = g.dist;
    return r;
}

RSG_D bool pair_has_candidates(const Ctx& a, int p) {
    int k = a.pkind[p];
    return ((k == PK_BALL_MESH || k == PK_CAR_MESH) && a.cand_n[a.pair1[p] - OBJ_BALL] >= 0) || k == PK_CAR_BALL;
}

// car vs car: btCompoundCompoundCollisionAlgorithm (btCompoundCompoundCollisionAlgorithm.cpp:213-330)
// over each car's single box child, then btBoxBoxCollisionAlgorithm with its own manifold.  The
// pair's algorithm runs with the later-added car as body 0.
RSG_DN void car_car_pair(const BatchView& bv, Ctx& a, int o0, int o1) {
    int ca = o1, cb = o0;
    Car& c0 = a.cars[ca - OBJ_CAR0];
    Car& c1 = a.cars[cb - OBJ_CAR0];
    V3 h0 = car_he(c0) + V3(c0.cfg->margin, c0.cfg->margin, c0.cfg->margin);
    V3 h1 = car_he(c1) + V3(c1.cfg->margin, c1.cfg->margin, c1.cfg->margin);
    Xf l0 = xf_identity(), l1 = xf_identity();
    l0.o = V3(c0.cfg->off[0], c0.cfg->off[1], c0.cfg->off[2]);
    l1.o = V3(c1.cfg->off[0], c1.cfg->off[1], c1.cfg->off[2]);
    V3 amn, amx, bmn, bmx, rmn, rmx;
    transform_aabb(car_he(c0), c0.cfg->margin, l0, amn, amx);
    transform_aabb(car_he(c1), c1.cfg->margin, l1, bmn, bmx);
    Xf rel = xf_mul(xf_inverse(c0.rb.xf), c1.rb.xf);
    transform_aabb_mm(bmn, bmx, rel, rmn, rmx);
    bool root = (amn.x <= rmx.x) && (amx.x >= rmn.x) && (amn.y <= rmx.y) && (amx.y >= rmn.y) && (amn.z <= rmx.z) &&
                (amx.z >= rmn.z);
    if (!root) return;
    Xf w0, w1;
    car_child_xf(c0, w0);
    car_child_xf(c1, w1);
    V3 m0, x0v, m1, x1v;
    car_box_aabb(c0, w0, m0, x0v);
    car_box_aabb(c1, w1, m1, x1v);
    if (!aabb_overlap(m0, x0v, m1, x1v)) return;
    float br = c0.cfg->breaking < c1.cfg->breaking ? c0.cfg->breaking : c1.cfg->breaking;
    Manifold& m = new_manifold(a, ca, cb, br);
    V3 nrm;
    BoxHit hits[4];
    int nh = box_box(w0.o, w0.b, h0, w1.o, w1.b, h1, nrm, hits);
    float fr = combined_friction(a, ca, cb), re = combined_restitution(a, ca, cb);
    for (int k = 0; k < nh; k++) {
        int idx = add_point(a, m, c0.rb.xf, c1.rb.xf, -nrm, hits[k].point, -hits[k].depth, fr, re);
        if (idx >= 0) contact_added(bv, a, m, idx, -1);
    }
    refresh(a, m, c0.rb.xf, c1.rb.xf);
}

// Lane 0's walk over the pairs in order (btCollisionDispatcher::dispatchAllCollisionPairs): pairs
// without candidates are processed when reached; a pair with candidates takes their results as
// the rounds deliver them.
struct CommitState {
    int p, j, mi;
    Xf x0, x1;
    float fr, re;
};
RSG_DN void commit_sweep(const BatchView& bv, Ctx& a, CommitState& cs, int base, int f_end) {
    while (cs.p < a.npairs) {
        const int p = cs.p, k = a.pkind[p];
        const int o0 = a.pair0[p], o1 = a.pair1[p];
        if (!pair_has_candidates(a, p)) {
            if (k == PK_BALL_MESH || k == PK_CAR_MESH) {  // more candidates than a segment holds
                Xf xf;
                Convex sh;
                float br;
                dyn_shape(a, o1, xf, sh, br);
                Manifold& m = new_manifold(a, o1, o0, br);
                convex_vs_mesh(bv, a, m, o1, xf, sh);
            } else if (k == PK_BALL_PLANE || k == PK_CAR_PLANE) {
                Xf xf;
                Convex sh;
                float br;
                dyn_shape(a, o1, xf, sh, br);
                Manifold& m = new_manifold(a, o1, o0, br);
                convex_vs_plane(bv, a, m, xf, sh, o0);
            } else if (k == PK_CAR_CAR) {
                car_car_pair(bv, a, o0, o1);
            }
            cs.p++;
            continue;
        }
        const int n = a.flat_n[p];
        if (cs.j == 0) {
            if (k == PK_CAR_BALL) {
                float cb = a.cars[o1 - OBJ_CAR0].cfg->breaking;
                cs.mi = a.nman;
                new_manifold(a, o1, OBJ_BALL, cb < a.ball_breaking ? cb : a.ball_breaking);
                cs.x0 = a.body(o1).xf;
                cs.x1 = a.ball.xf;
                cs.fr = combined_friction(a, OBJ_BALL, o1);
                cs.re = combined_restitution(a, OBJ_BALL, o1);
            } else {
                Xf xf;
                Convex sh;
                float br;
                dyn_shape(a, o1, xf, sh, br);
                cs.mi = a.nman;
                new_manifold(a, o1, o0, br);
                cs.x0 = a.body(o1).xf;
                cs.x1 = obj_xf(a, o0);
                cs.fr = combined_friction(a, OBJ_MESH, o1);
                cs.re = combined_restitution(a, OBJ_MESH, o1);
            }
        }
        Manifold& m = a.man[cs.mi];
        while (cs.j < n) {
            const int f = a.flat_off[p] + cs.j;
            if (f >= f_end) return;  // the next round delivers it
            const CandRes& r = a.cand_res[f - base];
            if (k == PK_CAR_BALL) {
                if (r.valid) {
                    int idx = add_point(a, m, cs.x0, cs.x1, r.n, r.p, r.d, cs.fr, cs.re);
                    if (idx >= 0) contact_added(bv, a, m, idx, -1);
                }
            } else {
                int t = a.cand_tri[(o1 - OBJ_BALL) * MESH_SEG + cs.j];
                commit_mesh_contact(bv, a, m, cs.x0, cs.x1, cs.fr, cs.re, r, t);
            }
            cs.j++;
        }
        refresh(a, m, cs.x0, cs.x1);
        cs.p++;
        cs.j = 0;
    }
}

RSG_DN void step_collide_tail(const BatchView& bv, Ctx& a);

// The first part of a world step's collision work on one arena's warp: the pair list, the BVH
// subtree headers and candidate triangles of each mesh pair, and the flattened candidate list.  Every
// warp of the block calls it, `active` or not; its parts are warp-local (block barriers between them
// measured 1-2 % slower).
RSG_DN void step_collide_gather(const BatchView& bv, Ctx& a, int lane, bool active) {
#if defined(RSG_PHASE_TIMERS)
    long long rsg_w_ = clock64();
#define RSG_W(i) do { if (lane == 0) { long long t_ = clock64(); atomicAdd(&g_phase_cycles[i], (unsigned long long)(t_ - rsg_w_)); rsg_w_ = t_; } } while (0)
#else
#define RSG_W(i)
#endif
    if (active) {
        build_pairs_warp(bv, a, lane);
        if (lane == 0) {
            a.nman = 0;
            a.npts = 0;
            a.warn = 0;
        }
    }
    __syncwarp();
    RSG_W(22);
    // quantized query box of each mesh pair (one lane per pair)
    unsigned qmask = 0;
    for (int p = lane; active && p < a.npairs; p += 32) {
        int k = a.pkind[p];
        if (k == PK_BALL_MESH || k == PK_CAR_MESH) {
            int d = a.pair1[p] - OBJ_BALL;
            Xf xf;
            Convex sh;
            float br;
            dyn_shape(a, a.pair1[p], xf, sh, br);
            V3 mn, mx;
            sh.aabb(xf, mn, mx);
            quantize_clamp(bv.mesh, a.qbox + d * 6, mn, false);
            quantize_clamp(bv.mesh, a.qbox + d * 6 + 3, mx, true);
            qmask |= 1u << d;
        }
    }
    qmask = __reduce_or_sync(0xffffffffu, qmask);
    __syncwarp();
    RSG_W(23);
    // subtree headers against every query box, 32 headers at a time; each query keeps the
    // overlapping headers in header order.  A run of 32 headers is scanned only for the queries
    // that overlap the box around the whole run.
    if (qmask) {
        int cnt[MAX_DYN];
        for (int d = 0; d < MAX_DYN; d++) cnt[d] = 0;
        const int nsub = bv.mesh.nsub, ngrp = bv.mesh.nsub_grp;
        for (int gbase = 0; gbase < ngrp; gbase += 32) {
            unsigned gm[MAX_DYN];
            {
                const int g = gbase + lane;
                uint16_t gmin[3], gmax[3];
                int gfirst = 0;
                if (g < ngrp) node_load_ptr(bv.mesh.sub_grp, g, gmin, gmax, gfirst);
                for (int d = 0; d < MAX_DYN; d++) {
                    gm[d] = 0;
                    if (!((qmask >> d) & 1u)) continue;
                    bool ov = g < ngrp && qov(a.qbox + d * 6, a.qbox + d * 6 + 3, gmin, gmax);
                    gm[d] = __ballot_sync(0xffffffffu, ov);
                }
            }
            unsigned any = 0;
            for (int d = 0; d < MAX_DYN; d++) any |= gm[d];
            while (any) {
                const int gi = __ffs(any) - 1;
                any &= any - 1;
                const int h = (gbase + gi) * 32 + lane;
                uint16_t smin[3], smax[3];
                int root = 0, size = 0;
                if (h < nsub) subtree_load_at(a.sub + h, smin, smax, root, size);
                for (int d = 0; d < MAX_DYN; d++) {
                    if (!((gm[d] >> gi) & 1u)) continue;
                    bool ov = h < nsub && qov(a.qbox + d * 6, a.qbox + d * 6 + 3, smin, smax);
                    unsigned m = __ballot_sync(0xffffffffu, ov);
                    if (ov) {
                        int pos = cnt[d] + __popc(m & ((1u << lane) - 1u));
                        if (pos < HDR_LIST) a.hdr_list[d * HDR_LIST + pos] = (int16_t)h;
                    }
                    cnt[d] += __popc(m);
                }
            }
        }
        if (lane == 0)
            for (int d = 0; d < MAX_DYN; d++)
                if ((qmask >> d) & 1u) a.hdr_n[d] = (int16_t)(cnt[d] <= HDR_LIST ? cnt[d] : -1);
    }
    __syncwarp();
    RSG_W(24);
    // candidate triangles of each mesh pair, one lane per pair, in BVH order
    for (int p = lane; active && p < a.npairs; p += 32) {
        int k = a.pkind[p];
        if (k == PK_BALL_MESH || k == PK_CAR_MESH) {
            int o = a.pair1[p];
            int d = o - OBJ_BALL;
            Xf xf;
            Convex sh;
            float br;
            dyn_shape(a, o, xf, sh, br);
            int* out = a.cand_tri + d * MESH_SEG;
            int n = 0;
            int nh = a.hdr_n[d];
            mesh_candidates(bv, xf, sh, br, a.sub, nh >= 0 ? a.hdr_list + d * HDR_LIST : nullptr, nh, [&](int t) {
                if (n < MESH_SEG) out[n] = t;
                n++;
            });
            a.cand_n[d] = (int16_t)(n <= MESH_SEG ? n : -1);
        }
    }
    __syncwarp();
    RSG_W(49);
    if (active && lane == 0) {
        int total = 0;
        for (int p = 0; p < a.npairs; p++) {
            int n = 0;
            if (pair_has_candidates(a, p)) n = a.pkind[p] == PK_CAR_BALL ? 1 : a.cand_n[a.pair1[p] - OBJ_BALL];
            a.flat_off[p] = (int16_t)total;
            a.flat_n[p] = (int16_t)n;
            total += n;
        }
        a.nflat = total;
    }
    __syncwarp();
}

// A world step's collision work (pairs, narrow phase, commits, islands, solver) for the arena of each
// warp of the block.  Every warp of the block calls it, `active` or not; with `bsync` the block's warps
// also meet at block-wide barriers between its parts (and between the test and commit halves of every
// round of candidate tests), so that they run the same code at the same time.
RSG_D void step_collide_block(const BatchView& bv, Ctx& a, int lane, bool active, bool bsync) {
    RSG_PHASE_BEGIN;
#if defined(RSG_PHASE_TIMERS)
    long long rsg_w_ = clock64();
#endif
    step_collide_gather(bv, a, lane, active);
    RSG_PHASE(4);
    if (bsync) __syncthreads();
    uint32_t warn = 0;
    // rounds of 32 candidate tests, then lane 0 commits them in pair order
    CommitState cs;
    cs.p = 0;
    cs.j = 0;
    cs.mi = 0;
    const int nflat = active ? a.nflat : 0;
    for (int base = 0; bsync ? __syncthreads_or(base < nflat) : (base < nflat); base += CAND_ROUND) {
        for (int f = base + lane; f < base + CAND_ROUND && f < nflat; f += 32) {
            int p = 0;
            while (!(f >= a.flat_off[p] && f < a.flat_off[p] + a.flat_n[p])) p++;
            const int o1 = a.pair1[p];
            if (a.pkind[p] == PK_CAR_BALL) {
                a.cand_res[f - base] = car_ball_test(a, o1, warn);
            } else {
                Xf xf;
                Convex sh;
                float br;
                dyn_shape(a, o1, xf, sh, br);
                int t = a.cand_tri[(o1 - OBJ_BALL) * MESH_SEG + (f - a.flat_off[p])];
                a.cand_res[f - base] = mesh_candidate_test(bv, xf, sh, br, t, warn);
            }
        }
        __syncwarp();
        RSG_W(46);
        if (bsync) __syncthreads();
        if (base < nflat && lane == 0)
            commit_sweep(bv, a, cs, base, base + CAND_ROUND < nflat ? base + CAND_ROUND : nflat);
        __syncwarp();
        RSG_W(47);
    }
    if (active) {
        if (warn) atomicOr(&a.warn, warn);
        __syncwarp();
        RSG_PHASE(5);
        if (lane == 0) {
            commit_sweep(bv, a, cs, nflat, nflat);
            a.err |= a.warn;
        }
        RSG_PHASE(6);
        if (lane == 0) step_collide_tail(bv, a);
        __syncwarp();
    }
    if (bsync) __syncthreads();
    if (active && a.solve_nb > 0) solve_setup_warp(a, lane, bv.dt);
    __syncwarp();
    if (bsync) __syncthreads();
    if (active && a.solve_nb > 0) solve_iterate_warp(a, lane, bv.dt);
    __syncwarp();
    RSG_PHASE(7);
}

// Register-array helpers for the at most MAX_DYN dynamic objects of an arena (unrolled selects
// keep the small arrays out of local memory).
RSG_D int rget(const int (&v)[MAX_DYN], int i) {
    int r = 0;
#pragma unroll
    for (int k = 0; k < MAX_DYN; k++) r = (k == i) ? v[k] : r;
    return r;
}
RSG_D void rset(int (&v)[MAX_DYN], int i, int x) {
#pragma unroll
    for (int k = 0; k < MAX_DYN; k++) v[k] = (k == i) ? x : v[k];
}

RSG_DN void step_collide_tail(const BatchView& bv, Ctx& a) {
    RSG_L0_BEGIN;
    const float dt = bv.dt;
    const int nd = 1 + a.ncars;
    RSG_L0(50);
    // per-body activation state and contact response, read once
    int act[MAX_DYN];
    unsigned resp = 0;
#pragma unroll
    for (int i = 0; i < MAX_DYN; i++) {
        act[i] = 0;
        if (i < nd) {
            const Body& b = a.body(OBJ_BALL + i);
            act[i] = b.act;
            if (!b.no_contact_response) resp |= 1u << i;
        }
    }
    // islands (btSimulationIslandManager, STATIC_SIMULATION_ISLAND_OPTIMIZATION): union by size
    // over the broadphase pairs in order
    RSG_L0(51);
    int tag[MAX_DYN];
#pragma unroll
    for (int i = 0; i < MAX_DYN; i++) tag[i] = i < nd ? i : -1;
    bool merging = false;  // any pair of two responding dynamic objects?
    for (int pi = 0; pi < a.npairs && !merging; pi++) {
        int p0 = a.pair0[pi];
        if (is_static_obj(p0)) continue;
        merging = ((resp >> (p0 - OBJ_BALL)) & 1u) && ((resp >> (a.pair1[pi] - OBJ_BALL)) & 1u);
    }
    if (merging) {
        int uf_id[MAX_DYN], uf_sz[MAX_DYN];
        for (int i = 0; i < nd; i++) { uf_id[i] = i; uf_sz[i] = 1; }
        auto find = [&](int x) { while (x != uf_id[x]) x = uf_id[x]; return x; };
        for (int pi = 0; pi < a.npairs; pi++) {
            int p0 = a.pair0[pi];
            if (is_static_obj(p0)) continue;
            int d0 = p0 - OBJ_BALL, d1 = a.pair1[pi] - OBJ_BALL;
            if (!((resp >> d0) & 1u) || !((resp >> d1) & 1u)) continue;
            int i = find(d0), j = find(d1);
            if (i == j) continue;
            if (uf_sz[i] < uf_sz[j]) { uf_id[i] = j; uf_sz[j] += uf_sz[i]; }
            else { uf_id[j] = i; uf_sz[i] += uf_sz[j]; }
        }
        int t[MAX_DYN];
        for (int i = 0; i < nd; i++) t[i] = find(i);
#pragma unroll
        for (int i = 0; i < MAX_DYN; i++)
            if (i < nd) tag[i] = t[i];
    }
    RSG_L0(52);
    // buildIslands: activation per island, island ids ascending
    if (!merging) {  // every body is its own island
#pragma unroll
        for (int i = 0; i < MAX_DYN; i++)
            if (i < nd && act[i] != ACTIVE_TAG && act[i] != DISABLE_DEACTIVATION && act[i] != DISABLE_SIMULATION)
                act[i] = ISLAND_SLEEPING;
    } else {
        int ta[MAX_DYN], aa[MAX_DYN];
        for (int i = 0; i < MAX_DYN; i++) { ta[i] = rget(tag, i); aa[i] = rget(act, i); }
        for (int id = 0; id < nd; id++) {
            bool present = false, all_sleeping = true;
            for (int i = 0; i < nd; i++)
                if (ta[i] == id) {
                    present = true;
                    if (aa[i] == ACTIVE_TAG || aa[i] == DISABLE_DEACTIVATION) all_sleeping = false;
                }
            if (!present) continue;
            for (int i = 0; i < nd; i++) {
                if (ta[i] != id) continue;
                if (all_sleeping) {
                    if (aa[i] != DISABLE_DEACTIVATION && aa[i] != DISABLE_SIMULATION) aa[i] = ISLAND_SLEEPING;
                } else if (aa[i] == ISLAND_SLEEPING) {
                    aa[i] = WANTS_DEACTIVATION;
                }
            }
        }
#pragma unroll
        for (int i = 0; i < MAX_DYN; i++) act[i] = aa[i];
    }
#pragma unroll
    for (int i = 0; i < MAX_DYN; i++)
        if (i < nd) a.body(OBJ_BALL + i).act = act[i];
    RSG_L0(53);
    // the tail's lists live in the candidate-triangle scratch, free once the narrow phase is done
    int* island_mans = a.cand_tri;
    int* solve_mans = island_mans + a.cap_pairs;
    int* qs_lo = solve_mans + a.cap_pairs;
    int* qs_hi = qs_lo + a.cap_pairs;
    int* bodies = qs_hi + a.cap_pairs;
    int nim = 0;
    for (int mi = 0; mi < a.nman; mi++) {
        Manifold& m = a.man[mi];
        const int b0 = m.body0, b1 = m.body1;
        const bool st0 = is_static_obj(b0), st1 = is_static_obj(b1);
        int s0 = st0 ? ISLAND_SLEEPING : rget(act, b0 - OBJ_BALL);
        int s1 = st1 ? ISLAND_SLEEPING : rget(act, b1 - OBJ_BALL);
        if (s0 != ISLAND_SLEEPING || s1 != ISLAND_SLEEPING) {
            bool r0 = st0 ? true : ((resp >> (b0 - OBJ_BALL)) & 1u);
            bool r1 = st1 ? true : ((resp >> (b1 - OBJ_BALL)) & 1u);
            if (r0 && r1 && (!st0 || !st1)) {
                int i0 = st0 ? -1 : rget(tag, b0 - OBJ_BALL);
                int i1 = st1 ? -1 : rget(tag, b1 - OBJ_BALL);
                m.island = (int8_t)(i0 >= 0 ? i0 : i1);
                island_mans[nim++] = mi;
            }
        }
    }
    RSG_L0(16);
    if (nim > 1) island_quicksort(a, island_mans, nim, qs_lo, qs_hi);
    RSG_L0(17);
    // processIslands: bodies and manifolds of awake islands, solved as one batch.  The sorted
    // manifold list is in island order, so one pass keeps each awake island's manifolds in order.
    unsigned awake = 0;
#pragma unroll
    for (int i = 0; i < MAX_DYN; i++)
        if (tag[i] >= 0 && act[i] != ISLAND_SLEEPING && act[i] != DISABLE_SIMULATION) awake |= 1u << tag[i];
    int nb = 0, nsm = 0;
    if (!merging) {  // island id == body index
        for (int i = 0; i < nd; i++)
            if ((awake >> i) & 1u) bodies[nb++] = OBJ_BALL + i;
    } else {
        for (int id = 0; id < nd; id++) {
            if (!((awake >> id) & 1u)) continue;
            for (int i = 0; i < nd; i++)
                if (rget(tag, i) == id) bodies[nb++] = OBJ_BALL + i;
        }
    }
    for (int k = 0; k < nim; k++)
        if ((awake >> a.man[island_mans[k]].island) & 1u) solve_mans[nsm++] = island_mans[k];
    a.solver_dt = dt;
    RSG_L0(18);
    a.solve_nb = 0;
    if (nb > 0) solve_plan(a, bodies, nb, solve_mans, nsm, bodies + MAX_DYN);
}

// Phase 3 of a world step, one lane per dynamic object: integration, activation, force reset.
RSG_D void step_bodies_post(const BatchView& bv, Ctx& a, int lane) {
    const float dt = bv.dt;
    const int nd = 1 + a.ncars;
    // integrateTransforms (btDiscreteDynamicsWorld.cpp:889-991)
    for (int d = lane; d < nd; d += 32) {
        Body& b = a.body(OBJ_BALL + d);
        if (b.is_active()) {
            Xf nt;
            integrate_transform(b.xf, b.lin_vel, b.ang_vel, dt, b.no_rot, nt);
            b.interp = nt;
            b.xf = nt;
            b.update_inertia();
        }
        // updateActivationState (btDiscreteDynamicsWorld.cpp:516-551).  The deactivation timer can
        // only move a body to WANTS_DEACTIVATION, which the next tick overwrites before anything
        // reads it, so it is not carried between ticks.
        if (b.act == ISLAND_SLEEPING || b.act == DISABLE_DEACTIVATION) {
        } else if (len2(b.lin_vel) < 0.8f * 0.8f && len2(b.ang_vel) < 1.f * 1.f) {
        } else {
            if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = 0;
        }
        bool wants = b.act != DISABLE_DEACTIVATION && (b.act == ISLAND_SLEEPING || b.act == WANTS_DEACTIVATION);
        if (wants) {
            if (b.act == ISLAND_SLEEPING) { b.ang_vel = V3(0, 0, 0); b.lin_vel = V3(0, 0, 0); }
        } else {
            if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = ACTIVE_TAG;
        }
        b.total_force = V3(0, 0, 0);  // clearForces
        b.total_torque = V3(0, 0, 0);
    }
}

// ---------------------------------------------------------------- boost pads and goal
RSG_D bool ball_scored(const Ctx& a, const MutatorsDev& m) {  // Arena::IsBallScored, soccar (src/Sim/Arena/Arena.cpp:893-901)
    float y = a.ball.xf.o.y * RL::BT_TO_UU;
    return fabsf(y) > (m.goal_threshold_y + m.ball_radius_uu);
}

// Arena::Step, one tick (src/Sim/Arena/Arena.cpp:689-756), run by the 32 lanes of one warp in four
// parts (tick_pre, step_bodies_pre, step_collide_warp, tick_post); the kernel puts a block-wide
// barrier between the parts so that the warps of a block run the same code at the same time.
//
// Work that is independent in the reference runs on separate lanes: the 16 suspension rays, the
// per-car logic after the rays, per-body integration and the boost pads.  Two situations make the
// cars depend on each other within the pre-tick, and then it runs car by car in update order
// like the reference: a car that is or just was demolished (its pre-tick changes its transform and
// collision response, which later cars' rays must see and earlier cars' rays must not), and a wheel
// resting on another car (its friction reads that car's velocity after that car's pre-tick).
// Collision detection, islands and the solver run on lane 0.
// The arenas of one block (one warp each), addressed by their index in the block.
struct BlockArenas {
    unsigned char* base;
    int bytes;  // shared memory per arena
    int nact;   // arenas of this block that exist
    RSG_D Ctx& operator()(int w) const { return *reinterpret_cast<Ctx*>(base + (size_t)w * bytes); }
};

// Thread `tid` of `nthreads` takes unit (tid % 32) * warps + tid / 32: consecutive units land in
// different warps.  Every unit count here is at most nthreads (32 wheel slots per arena).
RSG_D int spread_unit(int tid, int nthreads) { return (tid & 31) * (nthreads >> 5) + (tid >> 5); }

// Start of a tick for every arena of the block, the work spread over the block's threads by
// unit: arena, car, wheel, pad.  In the reference these run car by car; the units here are
// independent (a car's rays read only positions, cells and collision flags of other cars, none
// of which a pre-tick changes), except in the two situations that fall back to the reference's
// order for the whole arena: a car that is or just was demolished (its pre-tick moves it and
// changes its collision response, which earlier cars' rays must not see), and a wheel resting on
// another car (its friction reads that car's velocity after that car's pre-tick).
RSG_DN void block_tick_pre(const BatchView& bv, const BlockArenas& B, int tid, int nthreads) {
    const int MC = bv.MC;
    RSG_SUB_BEGIN;
    for (int w = tid; w < B.nact; w += nthreads) {
        Ctx& a = B(w);
        Body& ball = a.ball;
        bool ball_off = ball.act == DISABLE_DEACTIVATION || ball.act == DISABLE_SIMULATION;
        if (len2(ball.lin_vel) == 0 && len2(ball.ang_vel) == 0) {
            if (!ball_off) ball.act = ISLAND_SLEEPING;
        } else {
            if (!ball_off) ball.act = ACTIVE_TAG;
        }
        int serial = 0;
        for (int i = 0; i < a.ncars; i++) serial |= a.cars[i].f(F_DEMOED) || a.cars[i].rb.no_contact_response;
        a.serial = serial;
        a.on_car = 0;
    }
    __syncthreads();
    RSG_SUB(8);
    RSG_SUB(9);
    {  // one unit per wheel, spread over the block's warps: the wheel's transform and ray (an arena
       // in the reference's order runs its whole pre-tick on its first wheel's unit)
        const int u = spread_unit(tid, nthreads);
        Ctx& a = B(u / (MC * 4));
        int r = u % (MC * 4), k = r >> 2, wh = r & 3;
        if (u < B.nact * MC * 4 && a.serial && r == 0)
            for (int kk = 0; kk < a.ncars; kk++) car_pre_tick(bv, a, a.cars[a.order[kk]]);
        if (u < B.nact * MC * 4 && !a.serial && k < a.ncars) {
#if defined(RSG_PHASE_TIMERS)
        long long rt0_ = clock64();
#endif
        car_pre_before_rays_wheel(a.cars[k], wh);
        ray_cast_wheel(bv, a, a.cars[k], wh);
#if defined(RSG_PHASE_TIMERS)
        {
            long long dtw = clock64() - rt0_;
            atomicAdd(&g_phase_cycles[25], (unsigned long long)dtw);
            atomicAdd(&g_phase_cycles[26], 1ull);
            atomicMax(&g_phase_cycles[27], (unsigned long long)dtw);
        }
#endif
        if (a.cars[k].w[wh].ground >= OBJ_CAR0) a.on_car = 1;
        }
    }
    __syncthreads();
    RSG_SUB(10);
    {  // bv.lanes_per_car threads per car (1, 2 or 4; wheels split between them), cars spread over the warps
        const int LPC = bv.lanes_per_car;
        const int nw = nthreads >> 5, lane = tid & 31, g = lane / LPC, wl = lane % LPC;
        const int u = g * nw + (tid >> 5);
        const unsigned gmask = ((1u << LPC) - 1u) << (LPC * g);
        Ctx& a = B(u / MC);
        int k = u % MC;
        if (u < B.nact * MC && !a.serial && k < a.ncars) {
            if (a.on_car) {
                if (k == 0)
                    for (int kk = 0; kk < a.ncars; kk++) car_pre_after_rays_grp(bv, a, a.cars[a.order[kk]], wl, LPC, gmask);
            } else {
#if defined(RSG_PHASE_TIMERS)
                long long at0_ = clock64();
#endif
                car_pre_after_rays_grp(bv, a, a.cars[k], wl, LPC, gmask);
#if defined(RSG_PHASE_TIMERS)
                if (wl == 0) {
                    long long dtc = clock64() - at0_;
                    atomicAdd(&g_phase_cycles[28], (unsigned long long)dtc);
                    atomicAdd(&g_phase_cycles[29], 1ull);
                    atomicMax(&g_phase_cycles[30], (unsigned long long)dtc);
                }
#endif
            }
        }
    }
    if (bv.has_arena)
        for (int u = tid; u < B.nact * bv.npads; u += nthreads) {  // BoostPad::_PreTickUpdate (BoostPad.cpp:51-60)
            Ctx& a = B(u / bv.npads);
            if (a.ncars == 0) continue;
            Pad& p = a.pads[u % bv.npads];
            if (p.cooldown > 0) p.cooldown = rs_maxf(p.cooldown - bv.dt, 0);
            p.active = (p.cooldown == 0);
            p.cur_locked = -1;
        }
    __syncthreads();
    RSG_SUB(11);
}

// Body integration and activation (btDiscreteDynamicsWorld.cpp:516-551, 889-991) of one body.
RSG_DN void body_post(Body& b, float dt) {
    if (b.is_active()) {
        Xf nt;
        integrate_transform(b.xf, b.lin_vel, b.ang_vel, dt, b.no_rot, nt);
        b.interp = nt;
        b.xf = nt;
        b.update_inertia();
    }
    // The deactivation timer can only move a body to WANTS_DEACTIVATION, which the next tick
    // overwrites before anything reads it, so it is not carried between ticks.
    if (b.act == ISLAND_SLEEPING || b.act == DISABLE_DEACTIVATION) {
    } else if (len2(b.lin_vel) < 0.8f * 0.8f && len2(b.ang_vel) < 1.f * 1.f) {
    } else {
        if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = 0;
    }
    bool wants = b.act != DISABLE_DEACTIVATION && (b.act == ISLAND_SLEEPING || b.act == WANTS_DEACTIVATION);
    if (wants) {
        if (b.act == ISLAND_SLEEPING) { b.ang_vel = V3(0, 0, 0); b.lin_vel = V3(0, 0, 0); }
    } else {
        if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = ACTIVE_TAG;
    }
    b.total_force = V3(0, 0, 0);  // clearForces
    b.total_torque = V3(0, 0, 0);
}

// A pad's position (Bullet units), size and cell of BoostPadGrid (src/Sim/BoostPadGrid/BoostPadGrid.cpp:5-25),
// read from the batch's pad table (global memory: threads of a warp test different pads).
struct PadGeo {
    V3 pos_bt;
    int px, py;
    bool big;
};
RSG_D PadGeo pad_geo(const BatchView& bv, int pi) {
    const int CX = 8, CY = 10, SX = (int)(4096.f / (CX / 2)), SY = (int)(5120.f / (CY / 2));
    const float4 c = __ldg(bv.pad_cfg + pi);
    PadGeo g;
    g.px = (int)(c.x / SX + (CX / 2));
    g.py = (int)(c.y / SY + (CY / 2));
    g.pos_bt = V3(c.x, c.y, c.z) * RL::UU_TO_BT;
    g.big = c.w != 0.f;
    return g;
}

// BoostPadGrid::CheckCollision's early outs and the 3x3 cell neighbourhood of the car
RSG_D bool pad_grid_near(const Car& c, const PadGeo& g) {
    if (c.f(F_DEMOED) || c.boost >= RL::BOOST_MAX) return false;
    V3 cpu = c.rb.xf.o * RL::BT_TO_UU;
    const float EXT_Z = RL::PAD_CYL_HEIGHT + 250.f;
    if (cpu.z > EXT_Z) return false;
    const int CX = 8, CY = 10, SX = (int)(4096.f / (CX / 2)), SY = (int)(5120.f / (CY / 2));
    int ix = (int)(cpu.x / SX + (CX / 2));
    int iy = (int)(cpu.y / SY + (CY / 2));
    int i0 = ix - 1 > 0 ? ix - 1 : 0, i1 = ix + 1 < CX - 1 ? ix + 1 : CX - 1;
    int j0 = iy - 1 > 0 ? iy - 1 : 0, j1 = iy + 1 < CY - 1 ? iy + 1 : CY - 1;
    return !(g.px < i0 || g.px > i1 || g.py < j0 || g.py > j1);
}

// The pad test of one (pad, car): BoostPadGrid::CheckCollision's early outs and cell neighbourhood
// (src/Sim/BoostPadGrid/BoostPadGrid.cpp:5-25), then BoostPad::_CheckCollide (BoostPad.cpp:62-86).
// Custom pads skip the grid and its early outs (Arena.cpp:724-728).
RSG_D bool pad_touches(Ctx& a, const Pad& p, const PadGeo& g, int ci, bool custom) {
    Car& c = a.cars[ci];
    if (!custom && !pad_grid_near(c, g)) return false;
    const V3 cp = c.rb.xf.o;
    const V3 pos_bt = g.pos_bt;
    if (p.prev_locked == c.id) {
        V3 mn, mx;
        car_compound_aabb(c, c.rb.xf, mn, mx);
        float br = (g.big ? RL::PAD_BOX_RAD_BIG : RL::PAD_BOX_RAD_SMALL) * RL::UU_TO_BT;
        V3 bmin = pos_bt - V3(br, br, 0);
        V3 bmax = pos_bt + V3(br, br, RL::PAD_BOX_HEIGHT * RL::UU_TO_BT);
        bool gt = (bmax.x > mn.x) && (bmax.y > mn.y) && (bmax.z > mn.z);
        bool lt = (bmin.x < mx.x) && (bmin.y < mx.y) && (bmin.z < mx.z);
        return gt && lt;
    }
    float rad = (g.big ? RL::PAD_CYL_RAD_BIG : RL::PAD_CYL_RAD_SMALL) * RL::UU_TO_BT;
    float dx = cp.x - pos_bt.x, dy = cp.y - pos_bt.y;
    if (dx * dx + dy * dy < rad * rad) return fabsf(cp.z - pos_bt.z) < (RL::PAD_CYL_HEIGHT * RL::UU_TO_BT);
    return false;
}

// End of a tick for every arena of the block: integration, car post-ticks, boost pads, ball
// clamp, goal.  The pad pass of the reference (each car in update order marks the pads it
// touches, the last one wins; then each pad in order gives boost to its car) is done per pad
// and per car, which gives the same result because a pad's outcome depends only on the cars and
// a car's boost only on its pads taken in pad order.
// Tick end of one arena: Ball::_FinishPhysicsTick, the goal event, the tick counters.
RSG_D void arena_post(const BatchView& bv, Ctx& a) {
    Body& ball = a.ball;
    {  // Ball::_FinishPhysicsTick (src/Sim/Ball/Ball.cpp:117-143)
        if (!is_zero(a.ball_cache)) {
            ball.lin_vel += a.ball_cache;
            a.ball_cache = V3(0, 0, 0);
        }
        V3 v = ball.lin_vel, wv = ball.ang_vel;
        const float ms = bv.mut.ball_max_speed * RL::UU_TO_BT;
        if (len2(v) > ms * ms) v = normalized(v) * ms;
        if (len2(wv) > (RL::BALL_MAX_ANG_SPEED * RL::BALL_MAX_ANG_SPEED)) wv = normalized(wv) * RL::BALL_MAX_ANG_SPEED;
        ball.lin_vel = v;
        ball.ang_vel = wv;
        a.ball_ticks++;
    }
    if (bv.has_arena && ball_scored(a, bv.mut)) {
        uint32_t team = (-(a.ball.xf.o.y) < 0) ? 0u : 1u;  // RS_TEAM_FROM_Y(-y)
        push_event(a, RSG_EVENT_GOAL, team, 0, 0);
    }
    a.tick++;
    a.stepped = true;
}

RSG_DN void block_tick_post(const BatchView& bv, const BlockArenas& B, int tid, int nthreads) {
    RSG_SUB_BEGIN;
    const int MC = bv.MC, NB = MC + 1;
    for (int u = tid; u < B.nact * NB; u += nthreads) {
        Ctx& a = B(u / NB);
        int d = u % NB;
        if (d > a.ncars) continue;
        body_post(a.body(OBJ_BALL + d), bv.dt);
    }
    __syncthreads();
    RSG_SUB(12);
    for (int u = tid; u < B.nact * MC; u += nthreads) {
        Ctx& a = B(u / MC);
        int k = u % MC;
        if (k >= a.ncars) continue;
        car_post_tick(a.cars[k], bv.dt);
        car_finish_physics(a.cars[k]);
    }
    __syncthreads();
    RSG_SUB(13);
    if (bv.has_arena) {
        for (int u = tid; u < B.nact * bv.npads; u += nthreads) {  // which car each pad is locked to
            Ctx& a = B(u / bv.npads);
            int pi = u % bv.npads;
            Pad& p = a.pads[pi];
            const PadGeo g = pad_geo(bv, pi);
            for (int kk = 0; kk < a.ncars; kk++)
                if (pad_touches(a, p, g, a.order[kk], bv.custom_pads)) p.cur_locked = a.order[kk];
        }
        __syncthreads();
        for (int u = tid; u < B.nact * MC; u += nthreads) {  // BoostPad::_PostTickUpdate boost, in pad order
            Ctx& a = B(u / MC);
            int k = u % MC;
            if (k >= a.ncars) continue;
            Car& c = a.cars[k];
            for (int i = 0; i < bv.npads; i++) {
                const Pad& p = a.pads[i];
                if (p.cur_locked == k && p.active)
                    c.boost = rs_minf(c.boost + (__ldg(&bv.pad_cfg[i].w) != 0.f ? RL::PAD_BOOST_BIG : RL::PAD_BOOST_SMALL),
                                      RL::BOOST_MAX);
            }
        }
        __syncthreads();
        for (int u = tid; u < B.nact * bv.npads; u += nthreads) {  // BoostPad::_PostTickUpdate (BoostPad.cpp:88-105)
            Ctx& a = B(u / bv.npads);
            if (a.ncars == 0) continue;
            int i = u % bv.npads;
            Pad& p = a.pads[i];
            uint32_t locked = 0;
            if (p.cur_locked >= 0) {
                locked = a.cars[p.cur_locked].id;
                if (p.active) {
                    p.active = false;
                    p.cooldown = __ldg(&bv.pad_cfg[i].w) != 0.f ? bv.mut.pad_cooldown_big : bv.mut.pad_cooldown_small;
                }
            }
            p.prev_locked = locked;
        }
    }
    for (int w = tid; w < B.nact; w += nthreads) arena_post(bv, B(w));
    __syncthreads();
    RSG_SUB(14);
}

// ---------------------------------------------------------------- record load / store
RSG_D uint32_t pack_cell(int i, int j, int k) { return (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16); }

struct SoA {  // field accessors of one arena's record and scalars
    const BatchView& bv;
    int ar;
    RSG_D uint32_t* r() const { return bv.rec + (size_t)ar * bv.rec_words; }
    RSG_D float& cf(int f, int s) const { return reinterpret_cast<float*>(r())[rec_car_f(f, s)]; }
    RSG_D uint32_t& cu(int f, int s) const { return r()[rec_car_u(f, s)]; }
    RSG_D float& bf(int f) const { return reinterpret_cast<float*>(r())[rec_ball_f(f)]; }
    RSG_D uint32_t& bu(int f) const { return r()[rec_ball_u(f)]; }
    RSG_D float& pf(int f, int p) const { return reinterpret_cast<float*>(r())[rec_pad_f(f, p)]; }
    RSG_D uint32_t& pu(int f, int p) const { return r()[rec_pad_u(f, p)]; }
    RSG_D uint32_t& au(int f) const { return bv.au[(size_t)f * bv.A + ar]; }
    RSG_D V3 v3(int f, int s) const { return V3(cf(f, s), cf(f + 1, s), cf(f + 2, s)); }
    RSG_D void set_v3(int f, int s, V3 v) const { cf(f, s) = v.x; cf(f + 1, s) = v.y; cf(f + 2, s) = v.z; }
    RSG_D M3 m3(int f, int s) const {
        M3 m;
        for (int r_ = 0; r_ < 3; r_++) m.r[r_] = v3(f + 3 * r_, s);
        return m;
    }
    RSG_D void set_m3(int f, int s, const M3& m) const {
        for (int r_ = 0; r_ < 3; r_++) set_v3(f + 3 * r_, s, m.r[r_]);
    }
};

RSG_D void body_cell_load(const DevGrid& g, Body& b, uint32_t packed) {
    if (packed == 0xffffffffu) {
        b.cell = 0xffffffffu;
        b.ci = b.cj = b.ck = 0;
        return;
    }
    b.ci = (int)(packed & 0xff);
    b.cj = (int)((packed >> 8) & 0xff);
    b.ck = (int)((packed >> 16) & 0xff);
    b.cell = grid_cell_index(g, b.ci, b.cj, b.ck);
}
RSG_D uint32_t body_cell_store(const Body& b) { return b.cell == 0xffffffffu ? 0xffffffffu : pack_cell(b.ci, b.cj, b.ck); }

RSG_D void body_common(Body& b) {
    b.interp = b.xf;
    b.total_force = b.total_torque = V3(0, 0, 0);
    b.n_special = 0;
    b.sp_friction = b.sp_restitution = b.sp_total_dist = 0;
    b.sp_total_normal = V3(0, 0, 0);
    b.bp_min = b.bp_max = V3(0, 0, 0);
    b.update_inertia();
}

RSG_DN void load_arena(const BatchView& bv, int ar, Ctx& a) {  // scalars and ball (one lane)
    SoA s{bv, ar};
    a.ev = bv.events ? bv.events + (size_t)ar * MAX_EVENTS_PER_ARENA : nullptr;
    a.event_mask = bv.event_mask;
    a.tick = (uint64_t)s.au(AU_TICK_LO) | ((uint64_t)s.au(AU_TICK_HI) << 32);
    a.ncars = (int)s.au(AU_NCARS);
    uint32_t ord = s.au(AU_ORDER);
    for (int k = 0; k < MAX_CARS; k++) a.order[k] = (int)((ord >> (4 * k)) & 0xf);
    a.seq = s.au(AU_SEQ);
    a.stepped = s.au(AU_STEPPED) != 0;
    a.err = 0;
    a.nevents = (int)s.au(AU_EVENTS);
    a.solver_dt = a.stepped ? bv.dt : 1.f / 60.f;
    // ball (Ball::_BulletSetup, src/Sim/Ball/Ball.cpp:85-115)
    Body& b = a.ball;
    b.xf.o = V3(s.bf(BF_POS), s.bf(BF_POS + 1), s.bf(BF_POS + 2));
    for (int r = 0; r < 3; r++) b.xf.b.r[r] = V3(s.bf(BF_BASIS + 3 * r), s.bf(BF_BASIS + 3 * r + 1), s.bf(BF_BASIS + 3 * r + 2));
    b.lin_vel = V3(s.bf(BF_VEL), s.bf(BF_VEL + 1), s.bf(BF_VEL + 2));
    b.ang_vel = V3(s.bf(BF_ANG), s.bf(BF_ANG + 1), s.bf(BF_ANG + 2));
    a.ball_r = bv.mut.ball_radius_bt;
    a.ball_breaking = (a.ball_r + 0.08f) * 0.02f;  // getAngularMotionDisc * gContactBreakingThreshold
    {
        const float r = a.ball_r, mass = bv.mut.ball_mass;
        float elem = 0.4f * mass * r * r;
        b.inv_mass = 1.f / mass;
        b.inv_inertia_local = V3(1.f / elem, 1.f / elem, 1.f / elem);
    }
    b.lin_damping = bv.mut.ball_drag;
    b.act = ACTIVE_TAG;
    b.no_rot = bv.no_ball_rot != 0;
    b.no_contact_response = false;
    b.friction = bv.mut.ball_world_friction;
    b.restitution = bv.mut.ball_world_restitution;
    body_cell_load(bv.grid, b, s.bu(BU_CELL));
    b.cell_seq = s.bu(BU_CELL_SEQ);
    body_common(b);
    a.ball_ticks = (uint64_t)s.bu(BU_TICKS_LO) | ((uint64_t)s.bu(BU_TICKS_HI) << 32);
    a.ball_cache = V3(0, 0, 0);
    a.hs_dir = s.bf(BF_HS_DIR);
    a.hs_speed = s.bf(BF_HS_SPEED);
    a.hs_time = s.bf(BF_HS_TIME);
    // cars (Car::_BulletSetup, src/Sim/Car/Car.cpp:195-292, derived per config on the host)
}

RSG_DN void load_car(const BatchView& bv, int ar, Ctx& a, int i) {  // one car slot (one lane per car)
    SoA s{bv, ar};
    {
        Car& c = a.cars[i];
        c.cfg = bv.cfgs + s.cu(CU_CFG, i);
        c.obj = OBJ_CAR0 + i;
        c.flags = s.cu(CU_FLAGS, i);
        c.id = s.cu(CU_ID, i);
        c.cc_other = s.cu(CU_CC_OTHER, i);
        Body& rb = c.rb;
        rb.xf.o = s.v3(CF_POS, i);
        rb.xf.b = s.m3(CF_BASIS, i);
        rb.lin_vel = s.v3(CF_VEL, i);
        rb.ang_vel = s.v3(CF_ANG, i);
        rb.inv_mass = 1.f / RL::CAR_MASS_BT;
        rb.inv_inertia_local = V3(c.cfg->inv_inertia[0], c.cfg->inv_inertia[1], c.cfg->inv_inertia[2]);
        rb.lin_damping = 0;
        rb.no_rot = false;
        rb.no_contact_response = c.f(F_NO_RESPONSE);
        rb.act = rb.no_contact_response ? DISABLE_SIMULATION : ACTIVE_TAG;
        rb.friction = RL::CAR_COLLISION_FRICTION;
        rb.restitution = RL::CAR_COLLISION_RESTITUTION;
        body_cell_load(bv.grid, rb, s.cu(CU_CELL, i));
        rb.cell_seq = s.cu(CU_CELL_SEQ, i);
        body_common(rb);
        c.rot = s.m3(CF_ROT, i);
        c.steer = s.cf(CF_STEER, i);
        for (int w = 0; w < 4; w++) {
            c.pushback[w] = s.cf(CF_PUSHBACK + w, i);
            c.latf[w] = s.cf(CF_LATF + w, i);
            c.longf[w] = s.cf(CF_LONGF + w, i);
        }
        c.engine = s.cf(CF_ENGINE, i);
        c.brake = s.cf(CF_BRAKE, i);
        c.flip_rel = s.v3(CF_FLIP_REL, i);
        c.jump_time = s.cf(CF_JUMP_TIME, i);
        c.flip_time = s.cf(CF_FLIP_TIME, i);
        c.air_time = s.cf(CF_AIR_TIME, i);
        c.air_time_sj = s.cf(CF_AIR_TIME_SJ, i);
        c.boost = s.cf(CF_BOOST, i);
        c.time_since_boost = s.cf(CF_TIME_SINCE_BOOST, i);
        c.boosting_time = s.cf(CF_BOOSTING_TIME, i);
        c.supersonic_time = s.cf(CF_SUPERSONIC_TIME, i);
        c.handbrake = s.cf(CF_HANDBRAKE, i);
        c.autoflip_timer = s.cf(CF_AUTOFLIP_TIMER, i);
        c.autoflip_scale = s.cf(CF_AUTOFLIP_SCALE, i);
        c.wc_normal = s.v3(CF_WC_NORMAL, i);
        c.cc_cooldown = s.cf(CF_CC_COOLDOWN, i);
        c.demo_timer = s.cf(CF_DEMO_TIMER, i);
        c.bhi_rel = s.v3(CF_BHI_REL, i);
        c.bhi_ballpos = s.v3(CF_BHI_BALLPOS, i);
        c.bhi_extra = s.v3(CF_BHI_EXTRA, i);
        c.bhi_hit = (uint64_t)s.cu(CU_BHI_HIT_LO, i) | ((uint64_t)s.cu(CU_BHI_HIT_HI, i) << 32);
        c.bhi_extra_tick = (uint64_t)s.cu(CU_BHI_EXTRA_LO, i) | ((uint64_t)s.cu(CU_BHI_EXTRA_HI, i) << 32);
        c.ticks_since = (uint64_t)s.cu(CU_TICKS_LO, i) | ((uint64_t)s.cu(CU_TICKS_HI, i) << 32);
        for (int k = 0; k < 5; k++) {
            c.ctrl[k] = s.cf(CF_CTRL + k, i);
            c.last_ctrl[k] = s.cf(CF_LAST_CTRL + k, i);
        }
        c.vel_cache = s.v3(CF_VEL_CACHE, i);
    }
}

RSG_D void load_pads(const BatchView& bv, int ar, Ctx& a, int lane) {
    SoA s{bv, ar};
    for (int p = lane; p < NUM_PADS; p += 32) {
        Pad& pd = a.pads[p];
        pd.active = s.pu(PU_ACTIVE, p) != 0;
        pd.cooldown = s.pf(PF_COOLDOWN, p);
        pd.prev_locked = s.pu(PU_PREV_LOCKED, p);
        pd.cur_locked = (int)s.pu(PU_CUR_LOCKED, p) - 1;
    }
}

RSG_DN void store_arena(const BatchView& bv, int ar, Ctx& a) {
    SoA s{bv, ar};
    s.au(AU_TICK_LO) = (uint32_t)a.tick;
    s.au(AU_TICK_HI) = (uint32_t)(a.tick >> 32);
    s.au(AU_SEQ) = a.seq;
    s.au(AU_STEPPED) = a.stepped ? 1u : 0u;
    s.au(AU_ERR) |= a.err;
    s.au(AU_EVENTS) = (uint32_t)a.nevents;
    Body& b = a.ball;
    s.bf(BF_POS) = b.xf.o.x; s.bf(BF_POS + 1) = b.xf.o.y; s.bf(BF_POS + 2) = b.xf.o.z;
    for (int r = 0; r < 3; r++) {
        s.bf(BF_BASIS + 3 * r) = b.xf.b.r[r].x;
        s.bf(BF_BASIS + 3 * r + 1) = b.xf.b.r[r].y;
        s.bf(BF_BASIS + 3 * r + 2) = b.xf.b.r[r].z;
    }
    s.bf(BF_VEL) = b.lin_vel.x; s.bf(BF_VEL + 1) = b.lin_vel.y; s.bf(BF_VEL + 2) = b.lin_vel.z;
    s.bf(BF_ANG) = b.ang_vel.x; s.bf(BF_ANG + 1) = b.ang_vel.y; s.bf(BF_ANG + 2) = b.ang_vel.z;
    s.bu(BU_CELL) = body_cell_store(b);
    s.bu(BU_CELL_SEQ) = b.cell_seq;
    s.bu(BU_TICKS_LO) = (uint32_t)a.ball_ticks;
    s.bu(BU_TICKS_HI) = (uint32_t)(a.ball_ticks >> 32);
    s.bf(BF_HS_DIR) = a.hs_dir;
    s.bf(BF_HS_SPEED) = a.hs_speed;
    s.bf(BF_HS_TIME) = a.hs_time;
}

RSG_DN void store_car(const BatchView& bv, int ar, Ctx& a, int i) {
    SoA s{bv, ar};
    {
        Car& c = a.cars[i];
        c.setf(F_NO_RESPONSE, c.rb.no_contact_response);
        s.cu(CU_FLAGS, i) = c.flags;
        s.cu(CU_CC_OTHER, i) = c.cc_other;
        s.set_v3(CF_POS, i, c.rb.xf.o);
        s.set_m3(CF_BASIS, i, c.rb.xf.b);
        s.set_v3(CF_VEL, i, c.rb.lin_vel);
        s.set_v3(CF_ANG, i, c.rb.ang_vel);
        s.cu(CU_CELL, i) = body_cell_store(c.rb);
        s.cu(CU_CELL_SEQ, i) = c.rb.cell_seq;
        s.set_m3(CF_ROT, i, c.rot);
        s.cf(CF_STEER, i) = c.steer;
        for (int w = 0; w < 4; w++) {
            s.cf(CF_PUSHBACK + w, i) = c.pushback[w];
            s.cf(CF_LATF + w, i) = c.latf[w];
            s.cf(CF_LONGF + w, i) = c.longf[w];
        }
        s.cf(CF_ENGINE, i) = c.engine;
        s.cf(CF_BRAKE, i) = c.brake;
        s.set_v3(CF_FLIP_REL, i, c.flip_rel);
        s.cf(CF_JUMP_TIME, i) = c.jump_time;
        s.cf(CF_FLIP_TIME, i) = c.flip_time;
        s.cf(CF_AIR_TIME, i) = c.air_time;
        s.cf(CF_AIR_TIME_SJ, i) = c.air_time_sj;
        s.cf(CF_BOOST, i) = c.boost;
        s.cf(CF_TIME_SINCE_BOOST, i) = c.time_since_boost;
        s.cf(CF_BOOSTING_TIME, i) = c.boosting_time;
        s.cf(CF_SUPERSONIC_TIME, i) = c.supersonic_time;
        s.cf(CF_HANDBRAKE, i) = c.handbrake;
        s.cf(CF_AUTOFLIP_TIMER, i) = c.autoflip_timer;
        s.cf(CF_AUTOFLIP_SCALE, i) = c.autoflip_scale;
        s.set_v3(CF_WC_NORMAL, i, c.wc_normal);
        s.cf(CF_CC_COOLDOWN, i) = c.cc_cooldown;
        s.cf(CF_DEMO_TIMER, i) = c.demo_timer;
        s.set_v3(CF_BHI_REL, i, c.bhi_rel);
        s.set_v3(CF_BHI_BALLPOS, i, c.bhi_ballpos);
        s.set_v3(CF_BHI_EXTRA, i, c.bhi_extra);
        s.cu(CU_BHI_HIT_LO, i) = (uint32_t)c.bhi_hit;
        s.cu(CU_BHI_HIT_HI, i) = (uint32_t)(c.bhi_hit >> 32);
        s.cu(CU_BHI_EXTRA_LO, i) = (uint32_t)c.bhi_extra_tick;
        s.cu(CU_BHI_EXTRA_HI, i) = (uint32_t)(c.bhi_extra_tick >> 32);
        s.cu(CU_TICKS_LO, i) = (uint32_t)c.ticks_since;
        s.cu(CU_TICKS_HI, i) = (uint32_t)(c.ticks_since >> 32);
        for (int k = 0; k < 5; k++) {
            s.cf(CF_CTRL + k, i) = c.ctrl[k];
            s.cf(CF_LAST_CTRL + k, i) = c.last_ctrl[k];
        }
        s.set_v3(CF_VEL_CACHE, i, c.vel_cache);
    }
}

RSG_D void store_pads(const BatchView& bv, int ar, Ctx& a, int lane) {
    SoA s{bv, ar};
    for (int p = lane; p < NUM_PADS; p += 32) {
        Pad& pd = a.pads[p];
        s.pu(PU_ACTIVE, p) = pd.active ? 1u : 0u;
        s.pf(PF_COOLDOWN, p) = pd.cooldown;
        s.pu(PU_PREV_LOCKED, p) = pd.prev_locked;
        s.pu(PU_CUR_LOCKED, p) = (uint32_t)(pd.cur_locked + 1);
    }
}

// ---------------------------------------------------------------- shared-memory carve-out
// Byte offsets of one arena's working set inside its warp's shared-memory region.
struct SmemLayout {
    int cars, pads, pair0, pair1, man, pts, sb, rows_c, rows_f, pkind, flat_off, flat_n, cand_tri, cand_n, cand_res, qbox,
        hdr_list, hdr_n, bytes;
    int g_pts, g_rows, g_sb, g_cand, g_perm, g_bytes;  // parts in a per-warp global scratch (offsets, -1: shared)
    int perm;
    ArenaCaps caps;
};
RSG_HD int align16(int x) { return (x + 15) & ~15; }
// The manifold points and the solver rows live only within a tick's collision work; either can be
// kept in a global scratch of the warp (L1-cached) instead of shared memory.
RSG_HD SmemLayout smem_layout(int mc, bool rows_in_smem = true, bool pts_in_smem = true, bool more_in_smem = true) {
    SmemLayout L;
    L.caps = arena_caps(mc);
    L.g_pts = L.g_rows = L.g_sb = L.g_cand = L.g_perm = -1;
    const int perm_bytes = 2 * (2 * L.caps.rows + 2 * (MAX_DYN + 2));
    L.g_bytes = 0;
    const int cand_words = MESH_SEG * (mc + 1) > 4 * L.caps.pairs + MAX_DYN + L.caps.rows
                               ? MESH_SEG * (mc + 1)
                               : 4 * L.caps.pairs + MAX_DYN + L.caps.rows;
    if (!more_in_smem) {
        L.g_sb = L.g_bytes;
        L.g_bytes = align16(L.g_bytes + (int)sizeof(SBody) * (MAX_DYN + 1));
        L.g_cand = L.g_bytes;
        L.g_bytes = align16(L.g_bytes + 4 * cand_words);
        L.g_perm = L.g_bytes;
        L.g_bytes = align16(L.g_bytes + perm_bytes);
    }
    if (!pts_in_smem) {
        L.g_pts = L.g_bytes;
        L.g_bytes = align16(L.g_bytes + (int)sizeof(MPoint) * L.caps.points);
    }
    if (!rows_in_smem) {
        L.g_rows = L.g_bytes;
        L.g_bytes = align16(L.g_bytes + 2 * (int)sizeof(Row) * L.caps.rows);
    }
    int o = align16((int)sizeof(Ctx));
    L.cars = o;   o = align16(o + (int)sizeof(Car) * mc);
    L.pads = o;   o = align16(o + (int)sizeof(Pad) * NUM_PADS);
    L.pair0 = o;  o = align16(o + L.caps.pairs);
    L.pair1 = o;  o = align16(o + L.caps.pairs);
    L.man = o;    o = align16(o + (int)sizeof(Manifold) * L.caps.pairs);
    if (pts_in_smem) {
        L.pts = o; o = align16(o + (int)sizeof(MPoint) * L.caps.points);
    } else {
        L.pts = -1;
    }
    if (more_in_smem) {
        L.sb = o; o = align16(o + (int)sizeof(SBody) * (MAX_DYN + 1));
    } else {
        L.sb = -1;
    }
    if (rows_in_smem) {
        L.rows_c = o; o = align16(o + (int)sizeof(Row) * L.caps.rows);
        L.rows_f = o; o = align16(o + (int)sizeof(Row) * L.caps.rows);
    } else {
        L.rows_c = L.rows_f = -1;
    }
    L.pkind = o;  o = align16(o + L.caps.pairs);
    L.flat_off = o; o = align16(o + 2 * L.caps.pairs);
    L.flat_n = o; o = align16(o + 2 * L.caps.pairs);
    // candidate triangles; reused by the island / solver lists after the narrow phase
    if (more_in_smem) {
        L.cand_tri = o; o = align16(o + 4 * cand_words);
        L.perm = o; o = align16(o + perm_bytes);
    } else {
        L.cand_tri = L.perm = -1;
    }
    L.cand_n = o; o = align16(o + 2 * (mc + 1));
    L.cand_res = o; o = align16(o + (int)sizeof(CandRes) * CAND_ROUND);
    L.qbox = o; o = align16(o + 2 * 6 * MAX_DYN);
    L.hdr_list = o; o = align16(o + 2 * HDR_LIST * MAX_DYN);
    L.hdr_n = o; o = align16(o + 2 * MAX_DYN);
    L.bytes = o;
    return L;
}
// Lane 0 writes the carve-out pointers; the caller synchronises the warp before use.
// `gscr` is the warp's global scratch (L.g_bytes) for the parts the layout keeps out of shared memory.
RSG_D Ctx& bind_ctx(unsigned char* base, const SmemLayout& L, int lane, unsigned char* gscr = nullptr) {
    Ctx& a = *reinterpret_cast<Ctx*>(base);
    if (lane != 0) return a;
    a.cars = reinterpret_cast<Car*>(base + L.cars);
    a.pads = reinterpret_cast<Pad*>(base + L.pads);
    a.pair0 = reinterpret_cast<int8_t*>(base + L.pair0);
    a.pair1 = reinterpret_cast<int8_t*>(base + L.pair1);
    a.man = reinterpret_cast<Manifold*>(base + L.man);
    a.pts = reinterpret_cast<MPoint*>(L.pts >= 0 ? base + L.pts : gscr + L.g_pts);
    a.sb = reinterpret_cast<SBody*>(L.sb >= 0 ? base + L.sb : gscr + L.g_sb);
    a.rows_c = reinterpret_cast<Row*>(L.rows_c >= 0 ? base + L.rows_c : gscr + L.g_rows);
    a.rows_f = L.rows_c >= 0 ? reinterpret_cast<Row*>(base + L.rows_f) : a.rows_c + L.caps.rows;
    a.pkind = reinterpret_cast<int8_t*>(base + L.pkind);
    a.flat_off = reinterpret_cast<int16_t*>(base + L.flat_off);
    a.flat_n = reinterpret_cast<int16_t*>(base + L.flat_n);
    a.cand_tri = reinterpret_cast<int*>(L.cand_tri >= 0 ? base + L.cand_tri : gscr + L.g_cand);
    a.solve_perm = reinterpret_cast<int16_t*>(L.perm >= 0 ? base + L.perm : gscr + L.g_perm);
    a.cand_n = reinterpret_cast<int16_t*>(base + L.cand_n);
    a.cand_res = reinterpret_cast<CandRes*>(base + L.cand_res);
    a.qbox = reinterpret_cast<uint16_t*>(base + L.qbox);
    a.hdr_list = reinterpret_cast<int16_t*>(base + L.hdr_list);
    a.hdr_n = reinterpret_cast<int16_t*>(base + L.hdr_n);
    a.cap_pairs = L.caps.pairs;
    a.cap_pts = L.caps.points;
    a.cap_rows = L.caps.rows;
    return a;
}

}  // namespace rsg
