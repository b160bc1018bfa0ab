// rs_oracle.cpp -- CPU restatement of RocketSim v2.2's Arena::Step (soccar).
//
// TEST ORACLE ONLY (see rs_oracle.h).  Each block cites the reference file and
// lines it restates; paths are relative to the RocketSim source tree, "B/" is
// libsrc/bullet3-3.24/.  The restatement keeps Bullet's bookkeeping where it
// decides results: pair order of the voxel broadphase, manifold creation order,
// island sorting (Bullet's own quicksort), solver row order, 4-point manifolds.
#include "rs_oracle.h"
#include "rs_oracle_math.h"

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

using namespace rso;

namespace {

constexpr float UU_TO_BT = 1.f / 50.f;  // src/BulletLink.h:12-15
constexpr float BT_TO_UU = 50.f;

// ---------------------------------------------------------------- constants
// src/RLConst.h:9-166 (soccar subset used by the tick)
namespace RL {
constexpr float GRAVITY_Z = -650.f;
constexpr float ARENA_EXTENT_X = 4096, ARENA_HEIGHT = 2048;
constexpr float ARENA_COLLISION_BASE_FRICTION = 0.6f, ARENA_COLLISION_BASE_RESTITUTION = 0.3f;
constexpr float CAR_MASS_BT = 180.f, BALL_MASS_BT = CAR_MASS_BT / 6.f;
constexpr float CAR_COLLISION_FRICTION = 0.3f, CAR_COLLISION_RESTITUTION = 0.1f;
constexpr float CARBALL_COLLISION_FRICTION = 2.0f, CARBALL_COLLISION_RESTITUTION = 0.0f;
constexpr float CARWORLD_COLLISION_FRICTION = 0.3f, CARWORLD_COLLISION_RESTITUTION = 0.3f;
constexpr float CARCAR_COLLISION_FRICTION = 0.09f, CARCAR_COLLISION_RESTITUTION = 0.1f;
constexpr float BALL_REST_Z = 93.15f, BALL_MAX_ANG_SPEED = 6.f, BALL_DRAG = 0.03f;
constexpr float BALL_FRICTION = 0.35f, BALL_RESTITUTION = 0.6f;
constexpr float CAR_MAX_SPEED = 2300.f, BALL_MAX_SPEED = 6000.f;
constexpr float BOOST_MAX = 100.f, BOOST_USED_PER_SECOND = BOOST_MAX / 3, BOOST_MIN_TIME = 0.1f;
constexpr float BOOST_ACCEL_GROUND = 2975 / 3.f, BOOST_ACCEL_AIR = 3175 / 3.f, BOOST_SPAWN_AMOUNT = BOOST_MAX / 3;
constexpr float RECHARGE_BOOST_PER_SECOND = 10, RECHARGE_BOOST_DELAY = 0.25;
constexpr float CAR_MAX_ANG_SPEED = 5.5f;
constexpr float SUPERSONIC_START_SPEED = 2200.f, SUPERSONIC_MAINTAIN_MIN_SPEED = SUPERSONIC_START_SPEED - 100.f;
constexpr float SUPERSONIC_MAINTAIN_MAX_TIME = 1.f;
constexpr float POWERSLIDE_RISE_RATE = 5, POWERSLIDE_FALL_RATE = 2;
constexpr float THROTTLE_TORQUE_AMOUNT = CAR_MASS_BT * 400.f;
constexpr float BRAKE_TORQUE_AMOUNT = CAR_MASS_BT * (14.25f + (1.f / 3.f));
constexpr float STOPPING_FORWARD_VEL = 25.f, COASTING_BRAKE_FACTOR = 0.15f;
constexpr float BRAKING_NO_THROTTLE_SPEED_THRESH = 0.01f, THROTTLE_DEADZONE = 0.001f;
constexpr float THROTTLE_AIR_ACCEL = 200 / 3.f;
constexpr float JUMP_ACCEL = 4375.f / 3.f, JUMP_IMMEDIATE_FORCE = 875.f / 3.f, JUMP_MIN_TIME = 0.025f;
constexpr float JUMP_RESET_TIME_PAD = (1 / 40.f), JUMP_MAX_TIME = 0.2f, DOUBLEJUMP_MAX_DELAY = 1.25f;
constexpr float FLIP_Z_DAMP_120 = 0.35f, FLIP_Z_DAMP_START = 0.15f, FLIP_Z_DAMP_END = 0.21f;
constexpr float FLIP_TORQUE_TIME = 0.65f, FLIP_PITCHLOCK_EXTRA_TIME = 0.3f;
constexpr float FLIP_INITIAL_VEL_SCALE = 500.f, FLIP_TORQUE_X = 260.f, FLIP_TORQUE_Y = 224.f;
constexpr float FLIP_FORWARD_IMPULSE_MAX_SPEED_SCALE = 1.f, FLIP_SIDE_IMPULSE_MAX_SPEED_SCALE = 1.9f;
constexpr float FLIP_BACKWARD_IMPULSE_MAX_SPEED_SCALE = 2.5f, FLIP_BACKWARD_IMPULSE_SCALE_X = 16.f / 15.f;
constexpr float BALL_COLLISION_RADIUS_SOCCAR = 91.25f;
constexpr float SOCCAR_GOAL_SCORE_BASE_THRESHOLD_Y = 5124.25f;
constexpr float CAR_TORQUE_SCALE = 2 * 3.14159265358979323846 / (1 << 16) * 1000;
constexpr float CAR_AUTOFLIP_IMPULSE = 200, CAR_AUTOFLIP_TORQUE = 50, CAR_AUTOFLIP_TIME = 0.4f;
constexpr float CAR_AUTOFLIP_NORMZ_THRESH = 0.70710678118654752440, CAR_AUTOFLIP_ROLL_THRESH = 2.8f;
constexpr float CAR_AUTOROLL_FORCE = 100, CAR_AUTOROLL_TORQUE = 80;
constexpr float BALL_CAR_EXTRA_IMPULSE_Z_SCALE = 0.35f, BALL_CAR_EXTRA_IMPULSE_FORWARD_SCALE = 0.65f;
constexpr float BALL_CAR_EXTRA_IMPULSE_MAXDELTAVEL_UU = 4600.f;
constexpr float CAR_SPAWN_REST_Z = 17.f, CAR_RESPAWN_Z = 36.f;
constexpr float BUMP_COOLDOWN_TIME = 0.25f, BUMP_MIN_FORWARD_DIST = 64.5f, DEMO_RESPAWN_TIME = 3.f;
const V3 CAR_AIR_CONTROL_TORQUE(130, 95, 400), CAR_AIR_CONTROL_DAMPING(30, 20, 50);
namespace BTV {  // RLConst.h:156-166
constexpr float SUSPENSION_FORCE_SCALE_FRONT = 36.f - (1.f / 4.f);
constexpr float SUSPENSION_FORCE_SCALE_BACK = 54.f + (1.f / 4.f) + (1.5f / 100.f);
constexpr float SUSPENSION_STIFFNESS = 500.f, WHEELS_DAMPING_COMPRESSION = 25.f;
constexpr float WHEELS_DAMPING_RELAXATION = 40.f, MAX_SUSPENSION_TRAVEL = 12.f, SUSPENSION_SUBTRACTION = 0.05f;
}  // namespace BTV
namespace Pads {  // RLConst.h:250-310
constexpr float CYL_HEIGHT = 95, CYL_RAD_BIG = 208, CYL_RAD_SMALL = 144, BOX_HEIGHT = 64;
constexpr float BOX_RAD_BIG = 160, BOX_RAD_SMALL = 120, COOLDOWN_BIG = 10, COOLDOWN_SMALL = 4;
constexpr float BOOST_AMOUNT_BIG = 100, BOOST_AMOUNT_SMALL = 12;
const V3 LOCS_SMALL[28] = {
    {0.f, -4240.f, 70.f}, {-1792.f, -4184.f, 70.f}, {1792.f, -4184.f, 70.f}, {-940.f, -3308.f, 70.f},
    {940.f, -3308.f, 70.f}, {0.f, -2816.f, 70.f}, {-3584.f, -2484.f, 70.f}, {3584.f, -2484.f, 70.f},
    {-1788.f, -2300.f, 70.f}, {1788.f, -2300.f, 70.f}, {-2048.f, -1036.f, 70.f}, {0.f, -1024.f, 70.f},
    {2048.f, -1036.f, 70.f}, {-1024.f, 0.f, 70.f}, {1024.f, 0.f, 70.f}, {-2048.f, 1036.f, 70.f},
    {0.f, 1024.f, 70.f}, {2048.f, 1036.f, 70.f}, {-1788.f, 2300.f, 70.f}, {1788.f, 2300.f, 70.f},
    {-3584.f, 2484.f, 70.f}, {3584.f, 2484.f, 70.f}, {0.f, 2816.f, 70.f}, {-940.f, 3308.f, 70.f},
    {940.f, 3308.f, 70.f}, {-1792.f, 4184.f, 70.f}, {1792.f, 4184.f, 70.f}, {0.f, 4240.f, 70.f}};
const V3 LOCS_BIG[6] = {{-3584.f, 0.f, 73.f}, {3584.f, 0.f, 73.f}, {-3072.f, 4096.f, 73.f},
                        {3072.f, 4096.f, 73.f}, {-3072.f, -4096.f, 73.f}, {3072.f, -4096.f, 73.f}};
}  // namespace Pads
struct SpawnPos { float x, y, yaw; };
const SpawnPos RESPAWN_SOCCAR[4] = {{-2304, -4608, (float)(3.14159265358979323846 / 2)},
                                    {-2688, -4608, (float)(3.14159265358979323846 / 2)},
                                    {2304, -4608, (float)(3.14159265358979323846 / 2)},
                                    {2688, -4608, (float)(3.14159265358979323846 / 2)}};
}  // namespace RL

// LinearPieceCurve (src/Math/Math.cpp:5-35) over an ordered key list
struct Curve {
    int n;
    float x[6], y[6];
    float eval(float in, float def = 1) const {
        if (n == 0) return def;
        if (in <= x[0]) return y[0];
        for (int i = 1; i < n; i++) {
            if (x[i] > in) {
                float range = x[i] - x[i - 1];
                float diff = y[i] - y[i - 1];
                float f = (in - x[i - 1]) / range;
                return y[i - 1] + diff * f;
            }
        }
        return y[n - 1];
    }
};
// RLConst.h:388-490
const Curve STEER_ANGLE_FROM_SPEED = {6, {0, 500, 1000, 1500, 1750, 3000}, {0.53356f, 0.31930f, 0.18203f, 0.10570f, 0.08507f, 0.03454f}};
const Curve STEER_ANGLE_FROM_SPEED_THREEWHEEL = {2, {0, 2300}, {0.342473f, 0.034837f}};
const Curve POWERSLIDE_STEER_ANGLE_FROM_SPEED = {2, {0, 2500}, {0.39235f, 0.12610f}};
const Curve DRIVE_SPEED_TORQUE_FACTOR = {3, {0, 1400, 1410}, {1.0f, 0.1f, 0.0f}};
const Curve NON_STICKY_FRICTION_FACTOR = {3, {0, 0.7075f, 1}, {0.1f, 0.5f, 1.0f}};
const Curve LAT_FRICTION = {2, {0, 1}, {1.0f, 0.2f}};
const Curve LAT_FRICTION_THREEWHEEL = {2, {0, 1}, {0.30f, 0.25f}};
const Curve LONG_FRICTION = {0, {}, {}};
const Curve HANDBRAKE_LAT_FRICTION_FACTOR = {1, {0}, {0.1f}};
const Curve HANDBRAKE_LONG_FRICTION_FACTOR = {2, {0, 1}, {0.5f, 0.9f}};
const Curve BALL_CAR_EXTRA_IMPULSE_FACTOR = {4, {0, 500.f, 2300.f, 4600.f}, {0.65f, 0.65f, 0.55f, 0.30f}};
const Curve BUMP_VEL_AMOUNT_GROUND = {3, {0.f, 1400.f, 2200.f}, {(5.f / 6.f), 1100.f, 1530.f}};
const Curve BUMP_VEL_AMOUNT_AIR = {3, {0.f, 1400.f, 2200.f}, {(5.f / 6.f), 1390.f, 1945.f}};
const Curve BUMP_UPWARD_VEL_AMOUNT = {3, {0.f, 1400.f, 2200.f}, {(2.f / 6.f), 278.f, 417.f}};

// CarConfig presets, src/Sim/Car/CarConfig/CarConfig.cpp:20-99
struct Preset { V3 size, off; float frad, brad, fsus, bsus; V3 fwo, bwo; };
const Preset PRESETS[6] = {
    {{120.507f, 86.6994f, 38.6591f}, {13.8757f, 0, 20.755f}, 12.50f, 15.00f, 38.755f, 37.055f, {51.25f, 25.90f, 20.755f}, {-33.75f, 29.50f, 20.755f}},
    {{130.427f, 85.7799f, 33.8f}, {9.f, 0, 15.75f}, 12.00f, 13.50f, 33.95f, 33.85f, {50.30f, 31.10f, 15.75f}, {-34.75f, 33.00f, 15.75f}},
    {{131.32f, 87.1704f, 31.8944f}, {9.00857f, 0, 12.0942f}, 12.50f, 17.00f, 31.9242f, 27.9242f, {49.97f, 27.80f, 12.0942f}, {-35.43f, 20.28f, 12.0942f}},
    {{133.992f, 83.021f, 32.8f}, {12.5f, 0, 11.75f}, 13.50f, 15.00f, 29.7f, 29.666f, {51.50f, 26.67f, 11.75f}, {-35.75f, 35.00f, 11.75f}},
    {{129.519f, 84.6879f, 36.6591f}, {13.8757f, 0, 20.755f}, 12.50f, 15.00f, 38.755f, 37.055f, {51.25f, 25.90f, 20.755f}, {-34.00f, 29.50f, 20.755f}},
    {{123.22f, 79.2103f, 44.1591f}, {11.3757f, 0, 21.505f}, 15.00f, 15.00f, 39.505f, 39.105f, {51.25f, 25.90f, 21.505f}, {-33.75f, 29.50f, 21.505f}},
};

rsg_car_config preset_config(int i) {
    const Preset& p = PRESETS[i];
    rsg_car_config c;
    std::memset(&c, 0, sizeof(c));
    c.hitbox_size = {p.size.x, p.size.y, p.size.z};
    c.hitbox_pos_offset = {p.off.x, p.off.y, p.off.z};
    c.front_wheels.wheel_radius = p.frad;
    c.front_wheels.suspension_rest_length = p.fsus;
    c.front_wheels.connection_point_offset = {p.fwo.x, p.fwo.y, p.fwo.z};
    c.back_wheels.wheel_radius = p.brad;
    c.back_wheels.suspension_rest_length = p.bsus;
    c.back_wheels.connection_point_offset = {p.bwo.x, p.bwo.y, p.bwo.z};
    c.three_wheels = 0;
    c.dodge_deadzone = 0.5f;
    return c;
}

inline V3 V(const rsg_vec3& v) { return V3(v.x, v.y, v.z); }
inline rsg_vec3 P(V3 v) { return rsg_vec3{v.x, v.y, v.z}; }
inline float rs_max(float a, float b) { return (a > b) ? a : b; }  // RS_MAX (src/Framework.h)
inline float rs_min(float a, float b) { return (a < b) ? a : b; }
inline float rs_clamp(float v, float lo, float hi) { return rs_min(rs_max(v, lo), hi); }
inline int rs_sgn(float v) { return (v > 0) - (v < 0); }
// RocketSim's own Vec (src/Math/MathTypes/MathTypes.h:5-150): Length() guards 0,
// Normalized() divides (not multiplies by the reciprocal) and returns 0 below eps^2
inline float rs_len(V3 v) { float l2 = v.x * v.x + v.y * v.y + v.z * v.z; return l2 > 0 ? std::sqrt(l2) : 0.f; }
inline V3 rs_normalized(V3 v) {
    float l = rs_len(v);
    if (l > FLT_EPSILON * FLT_EPSILON) return V3(v.x / l, v.y / l, v.z / l);
    return V3(0, 0, 0);
}
// btSimdDot3 of the SSE2 solver rows (btSequentialImpulseConstraintSolver.cpp:104-108): x + (y + z)
inline float simd_dot(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }

// RotMat <-> btMatrix3x3: RotMat columns forward/right/up (MathTypes.h:169-185)
inline M3 rot_to_m3(const rsg_rotmat& r) {
    return M3(r.forward.x, r.right.x, r.up.x, r.forward.y, r.right.y, r.up.y, r.forward.z, r.right.z, r.up.z);
}
inline rsg_rotmat m3_to_rot(const M3& m) {
    rsg_rotmat r;
    r.forward = P(m.col(0));
    r.right = P(m.col(1));
    r.up = P(m.col(2));
    return r;
}

// ================================================================ mesh + BVH
// Quantized BVH, B/BulletCollision/BroadphaseCollision/btQuantizedBvh.cpp and
// B/BulletCollision/CollisionShapes/btOptimizedBvh.cpp:23-140
struct QNode {
    uint16_t qmin[3], qmax[3];
    int32_t esc_or_tri;  // >=0 triangle index (leaf), <0 -escape index
};
struct Subtree {
    uint16_t qmin[3], qmax[3];
    int root, size;
};
struct TriInfo {  // btTriangleInfo (B/.../CollisionShapes/btTriangleInfoMap.h:32-50)
    bool present = false;
    int flags = 0;
    float a01 = TWO_PI_F, a12 = TWO_PI_F, a20 = TWO_PI_F;
};
enum { TRI_V0V1_CONVEX = 1, TRI_V1V2_CONVEX = 2, TRI_V2V0_CONVEX = 4, TRI_V0V1_SWAP = 8, TRI_V1V2_SWAP = 16, TRI_V2V0_SWAP = 32 };

struct Mesh {
    std::vector<V3> verts;
    std::vector<int> tris;
    int ntri = 0;
    V3 aabb_min, aabb_max;  // local AABB (margin 0)
    V3 bvh_min, bvh_max, quant;
    std::vector<QNode> leaves, nodes;
    std::vector<Subtree> subtrees;
    int cur_node = 0;
    std::vector<TriInfo> info;

    void tri_verts(int t, V3 out[3]) const {
        for (int j = 0; j < 3; j++) out[j] = verts[tris[t * 3 + j]];
    }
    void quantize(uint16_t* out, V3 p, bool is_max) const {
        V3 v = (p - bvh_min) * quant;
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
    void quantize_clamp(uint16_t* out, V3 p, bool is_max) const {
        V3 c = vmin(vmax(p, bvh_min), bvh_max);
        quantize(out, c, is_max);
    }
    V3 unquantize(const uint16_t* q) const {
        V3 o((float)q[0] / quant.x, (float)q[1] / quant.y, (float)q[2] / quant.z);
        return o + bvh_min;
    }
    void set_quantization(V3 mn, V3 mx) {  // btQuantizedBvh::setQuantizationValues, margin 1
        V3 clampv(1.f, 1.f, 1.f);
        bvh_min = mn - clampv;
        bvh_max = mx + clampv;
        V3 size = bvh_max - bvh_min;
        quant = V3(65533.f / size.x, 65533.f / size.y, 65533.f / size.z);
        uint16_t q[3];
        quantize(q, bvh_min, false);
        V3 v = unquantize(q);
        bvh_min = vmin(bvh_min, v - clampv);
        size = bvh_max - bvh_min;
        quant = V3(65533.f / size.x, 65533.f / size.y, 65533.f / size.z);
        quantize(q, bvh_max, true);
        v = unquantize(q);
        bvh_max = vmax(bvh_max, v + clampv);
        size = bvh_max - bvh_min;
        quant = V3(65533.f / size.x, 65533.f / size.y, 65533.f / size.z);
    }
    V3 leaf_min(int i) const { return unquantize(leaves[i].qmin); }
    V3 leaf_max(int i) const { return unquantize(leaves[i].qmax); }
    int calc_split_axis(int s, int e) const {
        V3 means(0, 0, 0), variance(0, 0, 0);
        int n = e - s;
        for (int i = s; i < e; i++) means += 0.5f * (leaf_max(i) + leaf_min(i));
        means *= (1.f / (float)n);
        for (int i = s; i < e; i++) {
            V3 c = 0.5f * (leaf_max(i) + leaf_min(i));
            V3 d = c - means;
            d = d * d;
            variance += d;
        }
        variance *= (1.f / ((float)n - 1));
        return max_axis(variance);
    }
    int sort_split(int s, int e, int axis) {
        int split = s, n = e - s;
        V3 means(0, 0, 0);
        for (int i = s; i < e; i++) means += 0.5f * (leaf_max(i) + leaf_min(i));
        means *= (1.f / (float)n);
        float sv = means[axis];
        for (int i = s; i < e; i++) {
            V3 c = 0.5f * (leaf_max(i) + leaf_min(i));
            if (c[axis] > sv) {
                std::swap(leaves[i], leaves[split]);
                split++;
            }
        }
        int rb = n / 3;
        bool unbalanced = (split <= (s + rb)) || (split >= (e - 1 - rb));
        if (unbalanced) split = s + (n >> 1);
        return split;
    }
    void update_subtrees(int l, int r) {
        const int NODE = 16, MAXB = 2048;
        const QNode& ln = nodes[l];
        int lsz = ln.esc_or_tri >= 0 ? 1 : -ln.esc_or_tri;
        const QNode& rn = nodes[r];
        int rsz = rn.esc_or_tri >= 0 ? 1 : -rn.esc_or_tri;
        if (lsz * NODE <= MAXB) {
            Subtree st;
            std::memcpy(st.qmin, ln.qmin, 6); std::memcpy(st.qmax, ln.qmax, 6);
            st.root = l; st.size = lsz;
            subtrees.push_back(st);
        }
        if (rsz * NODE <= MAXB) {
            Subtree st;
            std::memcpy(st.qmin, rn.qmin, 6); std::memcpy(st.qmax, rn.qmax, 6);
            st.root = r; st.size = rsz;
            subtrees.push_back(st);
        }
    }
    void build_tree(int s, int e) {  // btQuantizedBvh::buildTree
        int n = e - s;
        int cur = cur_node;
        if (n == 1) {
            nodes[cur_node] = leaves[s];
            cur_node++;
            return;
        }
        int axis = calc_split_axis(s, e);
        int split = sort_split(s, e, axis);
        int internal = cur_node;
        quantize(nodes[internal].qmin, bvh_max, false);
        quantize(nodes[internal].qmax, bvh_min, true);
        for (int i = s; i < e; i++) {
            uint16_t qa[3], qb[3];
            quantize(qa, leaf_min(i), false);
            quantize(qb, leaf_max(i), true);
            for (int k = 0; k < 3; k++) {
                if (nodes[internal].qmin[k] > qa[k]) nodes[internal].qmin[k] = qa[k];
                if (nodes[internal].qmax[k] < qb[k]) nodes[internal].qmax[k] = qb[k];
            }
        }
        cur_node++;
        int left = cur_node;
        build_tree(s, split);
        int right = cur_node;
        build_tree(split, e);
        int esc = cur_node - cur;
        if (esc * 16 > 2048) update_subtrees(left, right);
        nodes[internal].esc_or_tri = -esc;
    }

    bool load(const uint8_t* data, uint64_t len) {  // CollisionMeshFile.cpp:11-73
        if (len < 8) return false;
        int32_t nt, nv;
        std::memcpy(&nt, data, 4);
        std::memcpy(&nv, data + 4, 4);
        if (std::min(nt, nv) <= 0 || std::max(nt, nv) > 1000000) return false;
        if ((uint64_t)8 + (uint64_t)nt * 12 + (uint64_t)nv * 12 > len) return false;
        tris.resize(nt * 3);
        std::memcpy(tris.data(), data + 8, (size_t)nt * 12);
        verts.resize(nv);
        const uint8_t* vp = data + 8 + (size_t)nt * 12;
        for (int i = 0; i < nv; i++) {
            float f[3];
            std::memcpy(f, vp + (size_t)i * 12, 12);
            verts[i] = V3(f[0], f[1], f[2]);
        }
        for (int i = 0; i < nt * 3; i++)
            if (tris[i] < 0 || tris[i] >= nv) return false;
        ntri = nt;
        // btTriangleMeshShape::recalcLocalAabb + btStridingMeshInterface::calculateAabbBruteForce
        V3 mn(BT_LARGE, BT_LARGE, BT_LARGE), mx(-BT_LARGE, -BT_LARGE, -BT_LARGE);
        for (int t = 0; t < nt; t++)
            for (int j = 0; j < 3; j++) {
                mn = vmin(mn, verts[tris[t * 3 + j]]);
                mx = vmax(mx, verts[tris[t * 3 + j]]);
            }
        aabb_min = mn;
        aabb_max = mx;
        set_quantization(mn, mx);
        leaves.resize(nt);
        for (int t = 0; t < nt; t++) {
            V3 tv[3];
            tri_verts(t, tv);
            V3 a(BT_LARGE, BT_LARGE, BT_LARGE), b(-BT_LARGE, -BT_LARGE, -BT_LARGE);
            for (int j = 0; j < 3; j++) { a = vmin(a, tv[j]); b = vmax(b, tv[j]); }
            const float MIN_DIM = 0.002f, MIN_HALF = 0.001f;
            for (int k = 0; k < 3; k++)
                if (b[k] - a[k] < MIN_DIM) { b[k] = b[k] + MIN_HALF; a[k] = a[k] - MIN_HALF; }
            quantize(leaves[t].qmin, a, false);
            quantize(leaves[t].qmax, b, true);
            leaves[t].esc_or_tri = t;
        }
        nodes.assign(2 * nt, QNode{});
        cur_node = 0;
        subtrees.clear();
        build_tree(0, nt);
        if (subtrees.empty()) {
            Subtree st;
            std::memcpy(st.qmin, nodes[0].qmin, 6); std::memcpy(st.qmax, nodes[0].qmax, 6);
            st.root = 0;
            st.size = nodes[0].esc_or_tri >= 0 ? 1 : -nodes[0].esc_or_tri;
            subtrees.push_back(st);
        }
        leaves.clear();
        build_edge_info();
        return true;
    }

    static bool qoverlap(const uint16_t* amin, const uint16_t* amax, const uint16_t* bmin, const uint16_t* bmax) {
        bool o = true;
        o = (amin[0] > bmax[0] || amax[0] < bmin[0]) ? false : o;
        o = (amin[2] > bmax[2] || amax[2] < bmin[2]) ? false : o;
        o = (amin[1] > bmax[1] || amax[1] < bmin[1]) ? false : o;
        return o;
    }
    // processAllTriangles with an AABB: walkStacklessQuantizedTreeCacheFriendly
    template <class F>
    void query_aabb(V3 mn, V3 mx, F&& f) const {
        uint16_t qa[3], qb[3];
        quantize_clamp(qa, mn, false);
        quantize_clamp(qb, mx, true);
        for (const Subtree& st : subtrees) {
            if (!qoverlap(qa, qb, st.qmin, st.qmax)) continue;
            int cur = st.root, end = st.root + st.size;
            while (cur < end) {
                const QNode& nd = nodes[cur];
                bool ov = qoverlap(qa, qb, nd.qmin, nd.qmax);
                bool leaf = nd.esc_or_tri >= 0;
                if (leaf && ov) f(nd.esc_or_tri);
                if (ov || leaf) cur++;
                else cur += -nd.esc_or_tri;
            }
        }
    }
    // reportRayOverlappingNodex: walkStacklessQuantizedTreeAgainstRay (btQuantizedBvh.cpp:436-548)
    template <class F>
    void query_ray(V3 src, V3 dst, F&& f) const {
        V3 dir = dst - src;
        dir = safe_normalized(dir);
        float lambda_max = dot(dir, dst - src);
        V3 inv(dir.x == 0.f ? BT_LARGE : 1.f / dir.x, dir.y == 0.f ? BT_LARGE : 1.f / dir.y,
               dir.z == 0.f ? BT_LARGE : 1.f / dir.z);
        unsigned sign[3] = {inv.x < 0.f, inv.y < 0.f, inv.z < 0.f};
        V3 rmin = vmin(src, dst), rmax = vmax(src, dst);
        uint16_t qa[3], qb[3];
        quantize_clamp(qa, rmin, false);
        quantize_clamp(qb, rmax, true);
        int cur = 0;
        while (cur < cur_node) {
            const QNode& nd = nodes[cur];
            bool rayov = false;
            bool boxov = qoverlap(qa, qb, nd.qmin, nd.qmax);
            bool leaf = nd.esc_or_tri >= 0;
            if (boxov) {
                V3 bounds[2] = {unquantize(nd.qmin), unquantize(nd.qmax)};
                float tmin, tmax, tymin, tymax, tzmin, tzmax;
                tmin = (bounds[sign[0]].x - src.x) * inv.x;
                tmax = (bounds[1 - sign[0]].x - src.x) * inv.x;
                tymin = (bounds[sign[1]].y - src.y) * inv.y;
                tymax = (bounds[1 - sign[1]].y - src.y) * inv.y;
                rayov = true;
                if ((tmin > tymax) || (tymin > tmax)) rayov = false;
                else {
                    if (tymin > tmin) tmin = tymin;
                    if (tymax < tmax) tmax = tymax;
                    tzmin = (bounds[sign[2]].z - src.z) * inv.z;
                    tzmax = (bounds[1 - sign[2]].z - src.z) * inv.z;
                    if ((tmin > tzmax) || (tzmin > tmax)) rayov = false;
                    else {
                        if (tzmin > tmin) tmin = tzmin;
                        if (tzmax < tmax) tmax = tzmax;
                        rayov = (tmin < lambda_max) && (tmax > 0.f);
                    }
                }
            }
            if (leaf && rayov) f(nd.esc_or_tri);
            if (rayov || leaf) cur++;
            else cur += -nd.esc_or_tri;
        }
    }

    // btGenerateInternalEdgeInfo, B/.../CollisionDispatch/btInternalEdgeUtility.cpp:33-305
    void build_edge_info() {
        info.assign(ntri, TriInfo{});
        const float EQV = 0.0001f * 0.0001f, PLANAR = 0.0001f;
        for (int ta = 0; ta < ntri; ta++) {
            V3 A[3];
            // vertices are fetched j = 2..0 in the reference; the values are the same
            tri_verts(ta, A);
            V3 mn(BT_LARGE, BT_LARGE, BT_LARGE), mx(-BT_LARGE, -BT_LARGE, -BT_LARGE);
            for (int j = 0; j < 3; j++) { mn = vmin(mn, A[j]); mx = vmax(mx, A[j]); }
            query_aabb(mn, mx, [&](int tb) {
                if (tb == ta) return;
                V3 B[3];
                tri_verts(tb, B);
                float crossB = len2(cross(B[1] - B[0], B[2] - B[0]));
                if (crossB < EQV) return;
                float crossA = len2(cross(A[1] - A[0], A[2] - A[0]));
                if (crossA < EQV) return;
                int numshared = 0, sa[3] = {-1, -1, -1}, sb[3] = {-1, -1, -1};
                for (int i = 0; i < 3; i++) {
                    for (int j = 0; j < 3; j++) {
                        if (len2(A[i] - B[j]) < EQV) {
                            sa[numshared] = i;
                            sb[numshared] = j;
                            numshared++;
                            if (numshared >= 3) return;
                        }
                    }
                    if (numshared >= 3) return;
                }
                if (numshared != 2) return;
                if (sa[0] == 0 && sa[1] == 2) {
                    sa[0] = 2; sa[1] = 0;
                    std::swap(sb[0], sb[1]);
                }
                TriInfo& inf = info[ta];
                inf.present = true;
                int sumA = sa[0] + sa[1];
                int otherA = 3 - sumA;
                V3 edge = A[sa[1]] - A[sa[0]];
                int otherB = 3 - (sb[0] + sb[1]);
                V3 tB0 = B[sb[1]], tB1 = B[sb[0]], tB2 = B[otherB];
                V3 normalA = normalized(cross(A[1] - A[0], A[2] - A[0]));
                V3 normalB = normalized(cross(tB1 - tB0, tB2 - tB0));
                edge = normalized(edge);
                V3 edgeCrossA = normalized(cross(edge, normalA));
                if (dot(edgeCrossA, A[otherA] - A[sa[0]]) < 0) edgeCrossA *= -1;
                V3 edgeCrossB = normalized(cross(edge, normalB));
                if (dot(edgeCrossB, B[otherB] - B[sb[0]]) < 0) edgeCrossB *= -1;
                float corrected = 0;
                bool isConvex = false;
                V3 calcEdge = cross(edgeCrossA, edgeCrossB);
                float l2 = len2(calcEdge);
                if (!(l2 < PLANAR)) {
                    calcEdge = normalized(calcEdge);
                    V3 calcNA = normalized(cross(calcEdge, edgeCrossA));
                    float angle2 = std::atan2(dot(edgeCrossB, calcNA), dot(edgeCrossB, edgeCrossA));
                    float ang4 = PI_F - angle2;
                    float dotA = dot(normalA, edgeCrossB);
                    isConvex = (dotA < 0.f);
                    corrected = isConvex ? ang4 : -ang4;
                }
                V3 e;
                int swapflag = 0, convflag = 0;
                float* ang = nullptr;
                if (sumA == 1) { e = A[0] - A[1]; swapflag = TRI_V0V1_SWAP; convflag = TRI_V0V1_CONVEX; ang = &inf.a01; }
                else if (sumA == 2) { e = A[2] - A[0]; swapflag = TRI_V2V0_SWAP; convflag = TRI_V2V0_CONVEX; ang = &inf.a20; }
                else { e = A[1] - A[2]; swapflag = TRI_V1V2_SWAP; convflag = TRI_V1V2_CONVEX; ang = &inf.a12; }
                Q orn = q_axis_angle(e, -corrected);
                V3 cnB = q_rotate(orn, normalA);
                if (dot(cnB, normalB) < 0) inf.flags |= swapflag;
                *ang = -corrected;
                if (isConvex) inf.flags |= convflag;
            });
        }
    }
};

std::unique_ptr<Mesh> g_mesh;
bool g_inited = false;

// ================================================================ broadphase grid
// btRSBroadphase (B/.../BroadphaseCollision/btRSBroadphase.cpp), ArenaConfig defaults
// (src/Sim/Arena/ArenaConfig/ArenaConfig.h:18-50): min (-5600,-6000,0) max (5600,6000,2200), cell 370 uu
struct Grid {
    V3 mn = V3(-5600, -6000, 0) * UU_TO_BT, mx = V3(5600, 6000, 2200) * UU_TO_BT;
    float cell = 370 * UU_TO_BT;
    int nx, ny, nz;
    std::vector<uint8_t> mesh_cells;  // 1 where the arena mesh is registered
    Grid() {
        V3 r = mx - mn;
        nx = std::max(1, (int)std::ceil(r.x / cell));
        ny = std::max(1, (int)std::ceil(r.y / cell));
        nz = std::max(1, (int)std::ceil(r.z / cell));
    }
    void indices(V3 p, int& i, int& j, int& k) const {
        V3 f = (p - mn) / cell;
        i = (int)f.x; j = (int)f.y; k = (int)f.z;
        i = std::min(std::max(i, 0), nx - 1);
        j = std::min(std::max(j, 0), ny - 1);
        k = std::min(std::max(k, 0), nz - 1);
    }
    int idx(int i, int j, int k) const { return i * ny * nz + j * nz + k; }
    V3 cell_min(int i, int j, int k) const { return mn + V3((float)i, (float)j, (float)k) * cell; }
    // _UpdateCellsStatic<true> for the mesh proxy (btRSBroadphase.cpp:71-140)
    void register_mesh(const Mesh& m, V3 amin, V3 amax) {
        mesh_cells.assign(nx * ny * nz, 0);
        V3 cmax = amax;
        for (int a = 0; a < 3; a++) cmax[a] = std::min(cmax[a], mx[a]);
        int i0, j0, k0, i1, j1, k1;
        indices(amin, i0, j0, k0);
        indices(cmax, i1, j1, k1);
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    V3 cmn = cell_min(i, j, k);
                    V3 cmx = cmn + V3(cell, cell, cell);
                    bool hit = false;
                    m.query_aabb(cmn, cmx, [&](int) { hit = true; });
                    if (!hit) continue;
                    for (int a = -1; a <= 1; a++)
                        for (int b = -1; b <= 1; b++)
                            for (int c = -1; c <= 1; c++) {
                                int ci = i + a, cj = j + b, ck = k + c;
                                if (ci < 0 || cj < 0 || ck < 0 || ci >= nx || cj >= ny || ck >= nz) continue;
                                mesh_cells[idx(ci, cj, ck)] = 1;
                            }
                }
    }
};
std::unique_ptr<Grid> g_grid;

// ================================================================ world objects
enum ActState { ACTIVE_TAG = 1, ISLAND_SLEEPING = 2, WANTS_DEACTIVATION = 3, DISABLE_DEACTIVATION = 4, DISABLE_SIMULATION = 5 };

struct Body {  // btRigidBody subset (B/BulletDynamics/Dynamics/btRigidBody.h)
    Xf xf, interp;
    V3 lin_vel, ang_vel, total_force, total_torque, gravity;
    float inv_mass = 0;
    V3 inv_inertia_local;
    M3 inv_inertia_world;
    float lin_damping = 0;
    bool no_rot = false;
    float friction = 0, restitution = 0;
    int act = ACTIVE_TAG;
    float deact_time = 0;
    bool no_contact_response = false;
    // broadphase proxy
    V3 bp_min, bp_max;
    int ci = 0, cj = 0, ck = 0, cell_idx = -1;
    uint64_t cell_seq = 0;
    // RocketSim special-contact accumulation (btCollisionObject.h:130)
    int n_special = 0;
    float sp_friction = 0, sp_restitution = 0, sp_total_dist = 0;
    V3 sp_total_normal;

    void update_inertia() { inv_inertia_world = scaled(xf.b, inv_inertia_local) * transpose(xf.b); }
    bool is_active() const { return act != ISLAND_SLEEPING && act != DISABLE_SIMULATION; }
    V3 vel_at(V3 rel) const { return lin_vel + cross(ang_vel, rel); }
    void apply_central_impulse(V3 imp) { lin_vel += imp * inv_mass; }
    void apply_torque_impulse(V3 t) { ang_vel += inv_inertia_world * t; }
    void apply_impulse(V3 imp, V3 rel) {
        if (inv_mass != 0.f) {
            apply_central_impulse(imp);
            apply_torque_impulse(cross(rel, imp));
        }
    }
    void apply_central_force(V3 f) { total_force += f; }
    void apply_torque(V3 t) { total_torque += t; }
    float impulse_denom(V3 pos, V3 n) const {  // btRigidBody::computeImpulseDenominator
        V3 r0 = pos - xf.o;
        V3 c0 = cross(r0, n);
        V3 vec = cross(c0 * inv_inertia_world, r0);
        return inv_mass + dot(n, vec);
    }
};

struct Wheel {  // btWheelInfoRL (src/Sim/btVehicleRL/btVehicleRL.h:9-27) + btWheelInfo
    V3 conn_cs, dir_cs = V3(0, 0, -1), axle_cs = V3(0, -1, 0);
    float rest_len = 0, travel_cm = 0, radius = 0;
    float stiffness = 0, damp_comp = 0, damp_relax = 0, force_scale = 0;
    bool front = false;
    // runtime (m_raycastInfo)
    V3 contact_normal, contact_point, hard_point, dir_ws, axle_ws;
    float susp_len = 0;
    bool in_contact = false;
    int ground = -1;  // collision object index of m_groundObject, -1 none
    M3 wbasis;
    float steer = 0, engine_force = 0, brake = 0;
    bool contact_world = false;
    V3 vel_at_contact;
    float lat_fric = 0, long_fric = 0;
    V3 impulse;
    float extra_pushback = 0, susp_rel_vel = 0, clipped_inv_dot = 0, susp_force = 0;
};

struct Car {
    uint32_t id = 0;
    int team = 0;
    rsg_car_config cfg;
    rsg_car_controls controls;
    rsg_car_state st;  // CarState mirror (pos/vel/angVel refreshed lazily, as the reference)
    Body rb;
    Wheel w[4];
    V3 hitbox_he;        // implicit shape dimensions (half extents minus margin)
    float hitbox_margin;  // btBoxShape margin after setSafeMargin
    V3 hitbox_off;
    V3 comp_min, comp_max;  // compound local AABB
    float breaking_threshold;
    V3 vel_impulse_cache;
    int obj = 0;  // collision object index
};

struct Pad {
    V3 pos_uu, pos_bt, box_min, box_max;
    bool big;
    bool active = true;
    float cooldown = 0;
    int cur_locked = -1;  // car index
    uint32_t prev_locked_id = 0;
};

struct MPoint {  // btManifoldPoint subset
    V3 local_a, local_b, pos_a, pos_b, normal;
    float dist = 0, friction = 0, restitution = 0;
    bool special = false;
};
struct Manifold {
    int body0, body1;  // collision object indices
    float breaking;
    int n = 0;
    MPoint pts[4];
    int island = -1;
};

// Collision object indices: [0] mesh, [1..4] floor, ceiling, wall -x, wall +x,
// [5] ball, [6..] cars in AddCar order (Arena.cpp:990-1068, 491-496, 50-62).
constexpr int OBJ_MESH = 0, OBJ_PLANE0 = 1, OBJ_BALL = 5, OBJ_CAR0 = 6;

struct Plane {
    V3 n;
    float c;  // plane constant (0); origin holds the position
    V3 origin;
    V3 aabb_min, aabb_max;  // broadphase AABB (with the contact threshold)
    V3 raw_min, raw_max;    // btStaticPlaneShape::getAabb
};

struct Event { uint32_t kind; uint64_t tick; uint32_t a, b, flag; };

struct Arena {
    int game_mode = 0;
    float tick_time = 1.f / 120.f;
    uint64_t tick_count = 0;
    uint32_t last_car_id = 0;
    float solver_dt = 1.f / 60.f;  // btContactSolverInfo::m_timeStep until the first world step
    Body ball;
    float ball_radius = RL::BALL_COLLISION_RADIUS_SOCCAR * UU_TO_BT;
    float ball_threshold;
    V3 ball_cache;
    uint64_t ball_ticks = 0;    // BallState::tickCountSinceUpdate
    std::vector<Car> cars;      // AddCar order
    std::vector<int> order;     // per-car update order (indices into cars)
    Pad pads[34];
    int npads = 0;
    Plane planes[4];
    bool has_arena = true;
    uint64_t cell_seq = 1;
    bool static_reg = false;  // statics re-registered by the first AABB update
    std::vector<Event> events;
    uint64_t counters[16] = {};
    V3 gravity;

    Body& body(int obj) { return obj == OBJ_BALL ? ball : cars[obj - OBJ_CAR0].rb; }
    bool is_static(int obj) const { return obj < OBJ_BALL; }
};

// ================================================================ setup
void setup_ball(Arena& a) {  // Ball::_BulletSetup (Ball.cpp:85-115), Arena.cpp:491-496
    Body& b = a.ball;
    float r = a.ball_radius;
    float mass = RL::BALL_MASS_BT;
    float elem = 0.4f * mass * r * r;
    b.inv_mass = 1.f / mass;
    b.inv_inertia_local = V3(1.f / elem, 1.f / elem, 1.f / elem);
    b.lin_damping = std::min(std::max(RL::BALL_DRAG, 0.f), 1.f);
    b.friction = RL::BALL_FRICTION;
    b.restitution = RL::BALL_RESTITUTION;
    b.no_rot = true;
    b.xf = xf_identity();
    b.xf.o = V3(0, 0, r);
    b.interp = b.xf;
    b.update_inertia();
    b.gravity = a.gravity * (1.f / b.inv_mass);
    a.ball_threshold = (r + 0.08f) * 0.02f;  // getAngularMotionDisc (btCollisionShape.cpp:128-150) * gContactBreakingThreshold
}

void set_ball_state(Arena& a, const rsg_ball_state& s) {  // Ball::SetState (Ball.cpp:35-51)
    Body& b = a.ball;
    b.xf.o = V(s.pos) * UU_TO_BT;
    b.xf.b = rot_to_m3(s.rot_mat);
    b.lin_vel = V(s.vel) * UU_TO_BT;
    b.ang_vel = V(s.ang_vel);
    b.update_inertia();
    if (!is_zero(V(s.vel)) || !is_zero(V(s.ang_vel))) {
        if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = ACTIVE_TAG;
    }
    a.ball_cache = V3(0, 0, 0);
    a.ball_ticks = 0;
}

void get_ball_state(Arena& a, rsg_ball_state& s) {
    std::memset(&s, 0, sizeof(s));
    s.tick_count_since_update = a.ball_ticks;
    s.pos = P(a.ball.xf.o * BT_TO_UU);
    s.rot_mat = m3_to_rot(a.ball.xf.b);
    s.vel = P(a.ball.lin_vel * BT_TO_UU);
    s.ang_vel = P(a.ball.ang_vel);
}

void setup_car(Arena& a, Car& c) {  // Car::_BulletSetup (Car.cpp:195-292)
    V3 size = V(c.cfg.hitbox_size);
    V3 he = (size * UU_TO_BT) / 2.f;
    // btBoxShape ctor + setSafeMargin (btBoxShape.cpp:17-25, btConvexInternalShape.h:63-90).
    // In this Bullet, setSafeMargin calls the non-virtual btConvexInternalShape::setMargin,
    // so the margin shrinks while the implicit (core) dimensions keep the 0.04 offset.
    float margin = 0.04f;
    V3 implicit = he - V3(margin, margin, margin);
    int minax = he.x < he.y ? (he.x < he.z ? 0 : 2) : (he.y < he.z ? 1 : 2);
    float safe = 0.1f * he[minax];
    if (safe < margin) margin = safe;
    c.hitbox_he = implicit;
    c.hitbox_margin = margin;
    c.hitbox_off = V(c.cfg.hitbox_pos_offset) * UU_TO_BT;
    V3 hm = implicit + V3(margin, margin, margin);
    c.comp_min = c.hitbox_off - hm;
    c.comp_max = c.hitbox_off + hm;
    // box inertia (btBoxShape.cpp:33-45) at CAR_MASS_BT
    float lx = 2.f * hm.x, ly = 2.f * hm.y, lz = 2.f * hm.z;
    float m = RL::CAR_MASS_BT;
    V3 inertia(m / 12.f * (ly * ly + lz * lz), m / 12.f * (lx * lx + lz * lz), m / 12.f * (lx * lx + ly * ly));
    Body& b = c.rb;
    b.inv_mass = 1.f / m;
    b.inv_inertia_local = V3(inertia.x != 0 ? 1.f / inertia.x : 0, inertia.y != 0 ? 1.f / inertia.y : 0,
                             inertia.z != 0 ? 1.f / inertia.z : 0);
    b.friction = RL::CAR_COLLISION_FRICTION;
    b.restitution = RL::CAR_COLLISION_RESTITUTION;
    b.xf = xf_identity();
    b.interp = b.xf;
    b.update_inertia();
    b.gravity = a.gravity * (1.f / b.inv_mass);
    // compound contact breaking threshold: getBoundingSphere from the local AABB
    V3 cmn = c.comp_min, cmx = c.comp_max;  // compound getAabb(identity), margin 0
    V3 lhe = 0.5f * (cmx - cmn), lc = 0.5f * (cmx + cmn);
    V3 amin = lc - lhe, amax = lc + lhe;
    float rad = len(amax - amin) * 0.5f;
    V3 cen = (amin + amax) * 0.5f;
    c.breaking_threshold = (rad + len(cen)) * 0.02f;
    // wheels (Car.cpp:235-289, btVehicleRL.cpp:34-57)
    for (int i = 0; i < 4; i++) {
        bool front = i < 2;
        bool left = i % 2;
        const rsg_wheel_pair_config& wp = front ? c.cfg.front_wheels : c.cfg.back_wheels;
        V3 off = V(wp.connection_point_offset);
        if (left) off.y *= -1;
        float rest = wp.suspension_rest_length - RL::BTV::MAX_SUSPENSION_TRAVEL;
        Wheel& w = c.w[i];
        w.conn_cs = off * UU_TO_BT;
        w.rest_len = rest * UU_TO_BT;
        w.radius = wp.wheel_radius * UU_TO_BT;
        w.stiffness = RL::BTV::SUSPENSION_STIFFNESS;
        w.damp_comp = RL::BTV::WHEELS_DAMPING_COMPRESSION;
        w.damp_relax = RL::BTV::WHEELS_DAMPING_RELAXATION;
        w.travel_cm = (RL::BTV::MAX_SUSPENSION_TRAVEL * UU_TO_BT) * 100;
        w.front = front;
        w.force_scale = front ? RL::BTV::SUSPENSION_FORCE_SCALE_FRONT : RL::BTV::SUSPENSION_FORCE_SCALE_BACK;
        w.steer = 0;
        w.extra_pushback = 0;
    }
}

void car_set_state(Car& c, const rsg_car_state& s) {  // Car::SetState (Car.cpp:23-36)
    c.rb.xf.o = V(s.pos) * UU_TO_BT;
    c.rb.xf.b = rot_to_m3(s.rot_mat);
    c.rb.lin_vel = V(s.vel) * UU_TO_BT;
    c.rb.ang_vel = V(s.ang_vel);
    c.rb.update_inertia();
    c.vel_impulse_cache = V3(0, 0, 0);
    c.st = s;
    c.st.tick_count_since_update = 0;
}

void car_refresh_state(Car& c) {  // Car::GetState (Car.cpp:10-20)
    c.st.pos = P(c.rb.xf.o * BT_TO_UU);
    c.st.vel = P(c.rb.lin_vel * BT_TO_UU);
    c.st.ang_vel = P(c.rb.ang_vel);
}

void car_respawn(Car& c, int idx, float boost) {  // Car::Respawn (Car.cpp:43-56)
    rsg_car_state s;
    std::memset(&s, 0, sizeof(s));
    const RL::SpawnPos& sp = RL::RESPAWN_SOCCAR[idx];
    s.pos = {sp.x, sp.y * (c.team == 0 ? 1 : -1), RL::CAR_RESPAWN_Z};
    float yaw = (float)(sp.yaw + (c.team == 0 ? 0 : 3.14159265358979323846));
    M3 m = m_euler_ypr(yaw, -0.f, -0.f);
    s.rot_mat = m3_to_rot(m);
    s.boost = boost;
    s.is_on_ground = 1;
    s.ball_hit_info.tick_count_when_hit = ~0ULL;
    s.ball_hit_info.tick_count_when_extra_impulse_applied = ~0ULL;
    car_set_state(c, s);
}

void setup_arena(Arena& a, int game_mode, float tick_rate) {  // Arena::Arena (Arena.cpp:416-540)
    a.game_mode = game_mode;
    a.tick_time = 1.f / tick_rate;
    a.has_arena = game_mode != RSG_GAMEMODE_THE_VOID;
    a.gravity = V3(0, 0, RL::GRAVITY_Z) * UU_TO_BT;
    // planes (Arena.cpp:1030-1068)
    const float H = RL::ARENA_HEIGHT, EX = RL::ARENA_EXTENT_X;
    V3 pos[4] = {V3(0, 0, 0), V3(0, 0, H), V3(-EX, 0, H / 2), V3(EX, 0, H / 2)};
    V3 nrm[4] = {V3(0, 0, 1), V3(0, 0, -1), V3(1, 0, 0), V3(-1, 0, 0)};
    for (int i = 0; i < 4; i++) {
        Plane& p = a.planes[i];
        p.n = normalized(nrm[i]);
        p.c = 0;
        p.origin = pos[i] * UU_TO_BT;
        // btStaticPlaneShape::getAabb (single-axis planes get a slab, btStaticPlaneShape.cpp:41-53)
        V3 mn(-BT_LARGE, -BT_LARGE, -BT_LARGE), mx(BT_LARGE, BT_LARGE, BT_LARGE);
        int ax = std::fabs(p.n.x) > 0.5f ? 0 : (std::fabs(p.n.y) > 0.5f ? 1 : 2);
        bool back = p.n[ax] < 0;
        mn[ax] = p.origin[ax] + (p.c - 0.2f);
        mx[ax] = p.origin[ax] + (p.c + 0.2f);
        (back ? mx : mn)[ax] = back ? BT_LARGE : -BT_LARGE;
        // broadphase AABBs carry the contact threshold (btCollisionWorld.cpp:143-150)
        p.raw_min = mn;
        p.raw_max = mx;
        p.aabb_min = mn - V3(0.02f, 0.02f, 0.02f);
        p.aabb_max = mx + V3(0.02f, 0.02f, 0.02f);
    }
    setup_ball(a);
    rsg_ball_state bs;
    std::memset(&bs, 0, sizeof(bs));
    bs.pos = {0, 0, RL::BALL_REST_Z};
    bs.rot_mat.forward = {1, 0, 0};
    bs.rot_mat.right = {0, 1, 0};
    bs.rot_mat.up = {0, 0, 1};
    set_ball_state(a, bs);
    a.ball.act = ACTIVE_TAG;
    a.ball.cell_seq = a.cell_seq++;
    // pads (Arena.cpp:498-534, BoostPad.cpp:37-49)
    a.npads = a.has_arena ? 34 : 0;
    for (int i = 0; i < a.npads; i++) {
        Pad& p = a.pads[i];
        p.big = i < 6;
        p.pos_uu = p.big ? RL::Pads::LOCS_BIG[i] : RL::Pads::LOCS_SMALL[i - 6];
        p.pos_bt = p.pos_uu * UU_TO_BT;
        float br = (p.big ? RL::Pads::BOX_RAD_BIG : RL::Pads::BOX_RAD_SMALL) * UU_TO_BT;
        p.box_min = p.pos_bt - V3(br, br, 0);
        p.box_max = p.pos_bt + V3(br, br, RL::Pads::BOX_HEIGHT * UU_TO_BT);
    }
}

// ================================================================ ray test
// btVehicleRL::rayCast -> btDefaultVehicleRaycaster::castRay -> btCollisionWorld::rayTest
// (btVehicleRL.cpp:120-209, btDefaultVehicleRaycaster.cpp:32-53, btCollisionWorld.cpp:257-545,877-966)
struct RayHit {
    bool hit = false;
    int obj = -1;
    float frac = 1.f;
    V3 normal, point;
};

// btTriangleRaycastCallback::processTriangle (B/.../NarrowPhaseCollision/btRaycastCallback.cpp:35-118)
inline bool ray_triangle(V3 from, V3 to, const V3 tv[3], float& hit_frac, V3& out_normal) {
    V3 v10 = tv[1] - tv[0], v20 = tv[2] - tv[0];
    V3 n = cross(v10, v20);
    float dist = dot(tv[0], n);
    float da = dot(n, from) - dist;
    float db = dot(n, to) - dist;
    if (da * db >= 0.f) return false;
    float proj = da - db;
    float distance = da / proj;
    if (!(distance < hit_frac)) return false;
    float tol = len2(n) * -0.0001f;
    V3 point = lerp(from, to, distance);
    V3 v0p = tv[0] - point, v1p = tv[1] - point;
    V3 cp0 = cross(v0p, v1p);
    if (!(dot(cp0, n) >= tol)) return false;
    V3 v2p = tv[2] - point;
    V3 cp1 = cross(v1p, v2p);
    if (!(dot(cp1, n) >= tol)) return false;
    V3 cp2 = cross(v2p, v0p);
    if (!(dot(cp2, n) >= tol)) return false;
    n = normalized(n);
    out_normal = (da <= 0.f) ? -n : n;
    hit_frac = distance;
    return true;
}

// btStaticPlaneShape::processAllTriangles (btStaticPlaneShape.cpp:56-87) fed to the ray callback
bool ray_plane(const Plane& p, V3 from_w, V3 to_w, float& hit_frac, V3& out_normal) {
    Xf t = xf_identity();
    t.o = p.origin;
    Xf inv = xf_inverse(t);
    V3 from = xf_apply(inv, from_w), to = xf_apply(inv, to_w);
    V3 amin = vmin(from, to), amax = vmax(from, to);
    V3 he = (amax - amin) * 0.5f;
    float radius = len(he);
    V3 center = (amax + amin) * 0.5f;
    V3 t0, t1;
    plane_space(p.n, t0, t1);
    V3 pc = center - (dot(p.n, center) - p.c) * p.n;
    bool any = false;
    V3 tri[3];
    tri[0] = pc + t0 * radius + t1 * radius;
    tri[1] = pc + t0 * radius - t1 * radius;
    tri[2] = pc - t0 * radius - t1 * radius;
    V3 nrm;
    if (ray_triangle(from, to, tri, hit_frac, nrm)) { any = true; out_normal = t.b * nrm; }
    tri[0] = pc - t0 * radius - t1 * radius;
    tri[1] = pc - t0 * radius + t1 * radius;
    tri[2] = pc + t0 * radius + t1 * radius;
    if (ray_triangle(from, to, tri, hit_frac, nrm)) { any = true; out_normal = t.b * nrm; }
    return any;
}

// Ray against the ball sphere / another car's box.  The reference uses
// btSubsimplexConvexCast, an iterative cast that converges to the same hit
// within its tolerance; this restatement solves the intersection directly.
bool ray_sphere(V3 from, V3 to, V3 c, float r, float& hit_frac, V3& out_normal) {
    V3 d = to - from, m = from - c;
    float a = dot(d, d), b = dot(m, d), cc = dot(m, m) - r * r;
    if (cc > 0.f && b > 0.f) return false;
    float disc = b * b - a * cc;
    if (disc < 0.f) return false;
    float t = (-b - std::sqrt(disc)) / a;
    if (t < 0.f) t = 0.f;
    if (!(t < hit_frac)) return false;
    V3 p = from + d * t;
    V3 n = p - c;
    if (len2(n) <= 0.0001f) return false;
    hit_frac = t;
    out_normal = normalized(n);
    return true;
}
bool ray_box(V3 from_w, V3 to_w, const Xf& box_xf, V3 he, float& hit_frac, V3& out_normal) {
    V3 from = xf_inv_apply(box_xf, from_w), to = xf_inv_apply(box_xf, to_w);
    V3 d = to - from;
    float tmin = 0.f, tmax = 1.f;
    int axis = -1;
    float sgn = 1;
    for (int k = 0; k < 3; k++) {
        if (std::fabs(d[k]) < 1e-12f) {
            if (from[k] < -he[k] || from[k] > he[k]) return false;
            continue;
        }
        float inv = 1.f / d[k];
        float t1 = (-he[k] - from[k]) * inv, t2 = (he[k] - from[k]) * inv;
        float s = -1;
        if (t1 > t2) { std::swap(t1, t2); s = 1; }
        if (t1 > tmin) { tmin = t1; axis = k; sgn = s; }
        if (t2 < tmax) tmax = t2;
        if (tmin > tmax) return false;
    }
    if (axis < 0) return false;
    if (!(tmin < hit_frac)) return false;
    V3 nl(0, 0, 0);
    nl[axis] = sgn;
    hit_frac = tmin;
    out_normal = box_xf.b * nl;
    return true;
}

bool dyn_registered_in(const Body& b, int ci, int cj, int ck) {
    return b.cell_idx >= 0 && std::abs(b.ci - ci) <= 1 && std::abs(b.cj - cj) <= 1 && std::abs(b.ck - ck) <= 1;
}

// dynamic proxies registered in a cell, in that cell's handle-list order
void cell_dyn_list(Arena& a, int ci, int cj, int ck, std::vector<int>& out) {
    out.clear();
    if (dyn_registered_in(a.ball, ci, cj, ck)) out.push_back(OBJ_BALL);
    for (size_t i = 0; i < a.cars.size(); i++)
        if (dyn_registered_in(a.cars[i].rb, ci, cj, ck)) out.push_back(OBJ_CAR0 + (int)i);
    std::stable_sort(out.begin(), out.end(), [&](int x, int y) { return a.body(x).cell_seq < a.body(y).cell_seq; });
}

// Ray against a dynamic object the way btCollisionWorld::rayTestSingleInternal casts it
// (btCollisionWorld.cpp:267-310): btSubsimplexConvexCast of a point against the car's box child
// (the car's compound has no child tree, Car.cpp:198) or the ball's sphere; defined after Simplex.
bool ray_cast_box(V3 from, V3 to, const Xf& box_xf, V3 he_margin, float& hit_frac, V3& out_normal);
bool ray_cast_sphere(V3 from, V3 to, const Xf& xf, float radius, float& hit_frac, V3& out_normal);

RayHit cast_ray(Arena& a, V3 from, V3 to, int self_obj) {
    RayHit r;
    float frac = 1.f;
    int obj = -1;
    V3 nrm;
    if (a.has_arena) {
        // static handles of the start cell: mesh, then the four planes
        const Mesh& m = *g_mesh;
        m.query_ray(from, to, [&](int t) {
            V3 tv[3];
            m.tri_verts(t, tv);
            V3 n;
            if (ray_triangle(from, to, tv, frac, n)) { obj = OBJ_MESH; nrm = n; }
        });
        for (int p = 0; p < 4; p++) {
            V3 n;
            if (ray_plane(a.planes[p], from, to, frac, n)) { obj = OBJ_PLANE0 + p; nrm = n; }
        }
    }
    int ci, cj, ck;
    g_grid->indices(from, ci, cj, ck);
    std::vector<int> dyn;
    cell_dyn_list(a, ci, cj, ck, dyn);
    for (int o : dyn) {
        if (o == self_obj) continue;
        if (frac == 0.f) break;
        V3 n;
        if (o == OBJ_BALL) {
            if (ray_cast_sphere(from, to, a.ball.xf, a.ball_radius, frac, n)) { obj = o; nrm = n; }
        } else {
            Car& c = a.cars[o - OBJ_CAR0];
            Xf bx = c.rb.xf;
            bx.o = xf_apply(c.rb.xf, c.hitbox_off);
            V3 he = c.hitbox_he + V3(c.hitbox_margin, c.hitbox_margin, c.hitbox_margin);
            if (ray_cast_box(from, to, bx, he, frac, n)) { obj = o; nrm = n; }
        }
    }
    if (obj < 0) return r;
    // castRay only accepts bodies with contact response (btDefaultVehicleRaycaster.cpp:40-51)
    if (!a.is_static(obj) && a.body(obj).no_contact_response) return r;
    r.hit = true;
    r.obj = obj;
    r.frac = frac;
    r.normal = normalized(nrm);
    r.point = lerp(from, to, frac);
    return r;
}

// ================================================================ vehicle
V3 chassis_up(const Car& c) { return c.rb.xf.b.col(2); }
V3 chassis_fwd(const Car& c) { return c.rb.xf.b.col(0); }

void wheel_transforms_ws(Car& c, Wheel& w) {  // btVehicleRL::updateWheelTransformsWS (btVehicleRL.cpp:110-118)
    w.in_contact = false;
    w.contact_world = false;
    w.hard_point = xf_apply(c.rb.xf, w.conn_cs);
    w.dir_ws = c.rb.xf.b * w.dir_cs;
    w.axle_ws = c.rb.xf.b * w.axle_cs;
}

void update_wheel_transform(Car& c, Wheel& w) {  // btVehicleRL::updateWheelTransform (btVehicleRL.cpp:66-94)
    wheel_transforms_ws(c, w);
    V3 up = -w.dir_ws;
    V3 right = w.axle_ws;
    V3 fwd = cross(up, right);
    fwd = normalized(fwd);
    Q so = q_axis_angle(up, w.steer);
    M3 sm = m_from_q(so);
    M3 b2;
    // right index 1, up index 2, forward index 0 (Car.cpp:243)
    for (int r = 0; r < 3; r++) {
        b2.r[r][1] = -right[r];
        b2.r[r][2] = up[r];
        b2.r[r][0] = fwd[r];
    }
    w.wbasis = sm * b2;
}

// resolveSingleCollision (B/BulletDynamics/ConstraintSolver/btContactConstraint.cpp:60-100), no impulse applied
float resolve_single_collision(Arena& a, Body& b1, int obj2, V3 pos, V3 n, float distance) {
    V3 rel1 = pos - b1.xf.o;
    bool dyn2 = !a.is_static(obj2);
    V3 o2 = dyn2 ? a.body(obj2).xf.o : (obj2 == OBJ_MESH ? V3(0, 0, 0) : a.planes[obj2 - OBJ_PLANE0].origin);
    V3 rel2 = pos - o2;
    V3 v1 = b1.vel_at(rel1);
    V3 v2 = dyn2 ? a.body(obj2).vel_at(rel2) : V3(0, 0, 0);
    V3 v = v1 - v2;
    float rel_vel = dot(n, v);
    float restitution = 0.f * -rel_vel;
    float pos_err = 0.2f * -distance / a.solver_dt;
    float vel_err = -(1.0f + restitution) * rel_vel;
    float d0 = b1.impulse_denom(pos, n);
    float d1 = dyn2 ? a.body(obj2).impulse_denom(pos, n) : 0.f;
    float jac = 1.f / (d0 + d1);
    float imp = pos_err * jac + vel_err * jac;
    imp = 0.f > imp ? 0.f : imp;
    return imp;
}

void ray_cast_wheel(Arena& a, Car& c, Wheel& w) {  // btVehicleRL::rayCast (btVehicleRL.cpp:120-209)
    wheel_transforms_ws(c, w);
    float travel = w.travel_cm / 100;
    float ray_len = w.rest_len + travel + w.radius - RL::BTV::SUSPENSION_SUBTRACTION;
    V3 src = w.hard_point;
    V3 dst = src + (w.dir_ws * ray_len);
    w.contact_point = dst;
    w.ground = -1;
    RayHit h = cast_ray(a, src, dst, c.obj);
    if (h.hit) {
        w.contact_point = h.point;
        w.contact_normal = h.normal;
        w.in_contact = true;
        bool stat = a.is_static(h.obj);
        w.contact_world = stat;
        w.ground = h.obj;
        V3 up = chassis_up(c);
        float trace = dot(w.hard_point - w.contact_point, up);
        w.susp_len = trace - w.radius;
        float lo = w.rest_len - travel, hi = w.rest_len + travel;
        w.susp_len = std::clamp(w.susp_len, lo, hi);
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
            float thresh = (w.rest_len + w.radius) - RL::BTV::SUSPENSION_SUBTRACTION;
            if (trace < thresh) {
                float delta = trace - thresh;
                float res = resolve_single_collision(a, c.rb, h.obj, h.point, h.normal, delta);
                w.extra_pushback = res / 4;
            }
        }
    } else {
        w.susp_len = w.rest_len + travel;
        w.susp_rel_vel = 0;
        w.contact_normal = -w.dir_ws;
        w.clipped_inv_dot = 1;
        w.extra_pushback = 0;
    }
}

// resolveSingleBilateral (btContactConstraint.cpp:103-150) with the btJacobianEntry diagonal
float resolve_single_bilateral(Arena& a, Body& b1, V3 pos1, int obj2, V3 pos2, V3 normal) {
    if (len2(normal) > 1.1f) return 0.f;
    bool dyn2 = !a.is_static(obj2);
    V3 o2 = dyn2 ? a.body(obj2).xf.o : (obj2 == OBJ_MESH ? V3(0, 0, 0) : a.planes[obj2 - OBJ_PLANE0].origin);
    V3 rel1 = pos1 - b1.xf.o;
    V3 rel2 = pos2 - o2;
    V3 v1 = b1.vel_at(rel1);
    V3 v2 = dyn2 ? a.body(obj2).vel_at(rel2) : V3(0, 0, 0);
    V3 v = v1 - v2;
    M3 w2a = transpose(b1.xf.b);
    M3 w2b = dyn2 ? transpose(a.body(obj2).xf.b) : M3();
    V3 aJ = w2a * cross(rel1, normal);
    V3 bJ = w2b * cross(rel2, -normal);
    V3 invIA = b1.inv_inertia_local;
    V3 invIB = dyn2 ? a.body(obj2).inv_inertia_local : V3(0, 0, 0);
    float invMB = dyn2 ? a.body(obj2).inv_mass : 0.f;
    V3 m0 = invIA * aJ, m1 = invIB * bJ;
    float diag = b1.inv_mass + dot(m0, aJ) + invMB + dot(m1, bJ);
    float jinv = 1.f / diag;
    float rel_vel = dot(normal, v);
    return -0.2f * rel_vel * jinv;
}

void calc_friction_impulses(Arena& a, Car& c, float dt) {  // btVehicleRL::calcFrictionImpulses (btVehicleRL.cpp:306-380)
    float fscale = (1.f / c.rb.inv_mass) / 3;
    for (int i = 0; i < 4; i++) {
        Wheel& w = c.w[i];
        if (w.ground >= 0) {
            V3 axle = w.wbasis.col(1);
            V3 n = w.contact_normal;
            float proj = dot(axle, n);
            axle -= n * proj;
            axle = safe_normalized(axle);
            V3 fwd = safe_normalized(cross(n, axle));
            float side = resolve_single_bilateral(a, c.rb, w.contact_point, w.ground, w.contact_point, axle);
            float roll;
            if (w.engine_force == 0) {
                if (w.brake) {
                    V3 cp = w.contact_point;
                    V3 crel = cp - c.rb.xf.o;
                    bool dyn2 = !a.is_static(w.ground);
                    V3 v1 = c.rb.vel_at(crel);
                    V3 v2 = dyn2 ? a.body(w.ground).vel_at(crel) : V3(0, 0, 0);
                    V3 cv = v1 - v2;
                    float rv = dot(cv, fwd);
                    if (dt > (1 / 80.f)) {
                        float th = -(1 / (dt * 150.f)) + 0.8f;
                        if (std::fabs(rv) < th) rv = 0;
                    }
                    const float MAGIC = 113.73963f;
                    roll = rs_clamp(-rv * MAGIC, -w.brake, w.brake);
                } else {
                    roll = 0;
                }
            } else {
                roll = -w.engine_force / fscale;
            }
            V3 total = (fwd * roll * w.long_fric) + (axle * side * w.lat_fric);
            w.impulse = total * fscale;
        } else {
            w.impulse = V3(0, 0, 0);
        }
    }
}

V3 upwards_from_wheels(const Car& c) {  // btVehicleRL::getUpwardsDirFromWheelContacts (btVehicleRL.cpp:397-410)
    V3 sum(0, 0, 0);
    for (int i = 0; i < 4; i++)
        if (c.w[i].in_contact) sum += c.w[i].contact_normal;
    if (sum == V3(0, 0, 0)) return chassis_up(c);
    return safe_normalized(sum);
}

void update_suspension(Car& c, float dt) {  // btVehicleRL::updateSuspension (btVehicleRL.cpp:270-303)
    for (int i = 0; i < 4; i++) {
        Wheel& w = c.w[i];
        if (w.in_contact) {
            float force = (w.rest_len - w.susp_len) * w.stiffness * w.clipped_inv_dot;
            float damp = (w.susp_rel_vel < 0) ? w.damp_comp : w.damp_relax;
            w.susp_force = force - (damp * w.susp_rel_vel);
            w.susp_force *= w.force_scale;
            if (w.susp_force < 0) w.susp_force = 0;
        } else {
            w.susp_force = 0;
        }
    }
    for (int i = 0; i < 4; i++) {
        Wheel& w = c.w[i];
        if (w.susp_force != 0) {
            V3 off = w.contact_point - c.rb.xf.o;
            float base = (w.susp_force * dt) + w.extra_pushback;
            V3 f = w.contact_normal * base;
            c.rb.apply_impulse(f, off);
        }
    }
}

void apply_friction_impulses(Car& c, float dt) {  // btVehicleRL::applyFrictionImpulses (btVehicleRL.cpp:383-395)
    V3 up = c.rb.xf.b.col(2);
    for (int i = 0; i < 4; i++) {
        Wheel& w = c.w[i];
        if (!is_zero(w.impulse)) {
            V3 off = w.contact_point - c.rb.xf.o;
            float d = dot(up, off);
            V3 rel = off - up * d;
            c.rb.apply_impulse(w.impulse * dt, rel);
        }
    }
}

// ================================================================ car logic (src/Sim/Car/Car.cpp)
inline V3 st_fwd(const Car& c) { return V(c.st.rot_mat.forward); }
inline V3 st_right(const Car& c) { return V(c.st.rot_mat.right); }
inline V3 st_up(const Car& c) { return V(c.st.rot_mat.up); }

void update_wheels(Car& c, float dt, int nwc, float fwd_speed) {  // Car::_UpdateWheels (Car.cpp:339-484)
    float absfs = std::fabs(fwd_speed);
    bool world_contact = false;
    for (int i = 0; i < 4; i++) world_contact |= c.w[i].contact_world;
    rsg_car_state& s = c.st;
    if (c.controls.handbrake) s.handbrake_val += RL::POWERSLIDE_RISE_RATE * dt;
    else s.handbrake_val -= RL::POWERSLIDE_FALL_RATE * dt;
    s.handbrake_val = rs_clamp(s.handbrake_val, 0, 1);
    float real_throttle = c.controls.throttle;
    float real_brake = 0;
    if (c.controls.boost && s.boost > 0) real_throttle = 1;
    {
        float dss = DRIVE_SPEED_TORQUE_FACTOR.eval(absfs);
        float eng = real_throttle;
        if (c.controls.handbrake) {
        } else {
            float at = std::fabs(real_throttle);
            if (at >= RL::THROTTLE_DEADZONE) {
                if (absfs > RL::STOPPING_FORWARD_VEL && rs_sgn(real_throttle) != rs_sgn(fwd_speed)) {
                    real_brake = 1;
                    if (absfs > RL::BRAKING_NO_THROTTLE_SPEED_THRESH) eng = 0;
                }
            } else {
                eng = 0;
                bool stop = (absfs < RL::STOPPING_FORWARD_VEL);
                real_brake = stop ? 1 : RL::COASTING_BRAKE_FACTOR;
            }
        }
        if (nwc < 3) dss /= 4;
        float ef = eng * (RL::THROTTLE_TORQUE_AMOUNT * UU_TO_BT) * dss;
        float bf = real_brake * (RL::BRAKE_TORQUE_AMOUNT * UU_TO_BT);
        for (int i = 0; i < 4; i++) { c.w[i].engine_force = ef; c.w[i].brake = bf; }
    }
    {
        float steer = (c.cfg.three_wheels ? STEER_ANGLE_FROM_SPEED_THREEWHEEL : STEER_ANGLE_FROM_SPEED).eval(absfs);
        if (s.handbrake_val) steer += (POWERSLIDE_STEER_ANGLE_FROM_SPEED.eval(absfs) - steer) * s.handbrake_val;
        steer *= c.controls.steer;
        c.w[0].steer = steer;
        c.w[1].steer = steer;
    }
    for (int i = 0; i < 4; i++) {
        Wheel& w = c.w[i];
        if (w.ground >= 0) {
            V3 vel = c.rb.lin_vel, av = c.rb.ang_vel;
            V3 lat = w.wbasis.col(1);
            V3 lng = cross(lat, w.contact_normal);
            float in = 0;
            V3 wd = w.hard_point - c.rb.xf.o;
            V3 cv = (cross(av, wd) + vel) * BT_TO_UU;
            float base = std::fabs(dot(cv, lat));
            if (base > 5) in = base / (std::fabs(dot(cv, lng)) + base);
            float latf = (c.cfg.three_wheels ? LAT_FRICTION_THREEWHEEL : LAT_FRICTION).eval(in);
            float longf = LONG_FRICTION.eval(in);
            if (s.handbrake_val) {
                float hb = s.handbrake_val;
                latf *= (HANDBRAKE_LAT_FRICTION_FACTOR.eval(in) - 1) * hb + 1;
                longf *= (HANDBRAKE_LONG_FRICTION_FACTOR.eval(in) - 1) * hb + 1;
            } else {
                longf = 1;
            }
            bool sticky = real_throttle != 0;
            if (!sticky) {
                float ns = NON_STICKY_FRICTION_FACTOR.eval(w.contact_normal.z);
                latf *= ns;
                longf *= ns;
            }
            w.lat_fric = latf;
            w.long_fric = longf;
        }
    }
    if (world_contact) {
        V3 updir = upwards_from_wheels(c);
        bool full = (real_throttle != 0) || (absfs > RL::STOPPING_FORWARD_VEL);
        float sfs = c.cfg.three_wheels ? 0 : 0.5f;
        if (full) sfs += 1 - std::fabs(updir.z);
        c.rb.apply_central_force(updir * sfs * (RL::GRAVITY_Z * UU_TO_BT) * RL::CAR_MASS_BT);
    }
}

void update_boost(Car& c, float dt) {  // Car::_UpdateBoost (Car.cpp:486-533)
    rsg_car_state& s = c.st;
    bool has = s.boost > 0;
    if (has) {
        if (s.is_boosting) s.is_boosting = (c.controls.boost || s.boosting_time < RL::BOOST_MIN_TIME);
        else if (c.controls.boost) s.is_boosting = 1;
    } else {
        s.is_boosting = 0;
    }
    if (s.is_boosting) s.boosting_time += dt;
    else s.boosting_time = 0;
    if (s.is_boosting) {
        s.boost = rs_max(s.boost - RL::BOOST_USED_PER_SECOND * dt, 0);
        c.rb.apply_central_force((s.is_on_ground ? RL::BOOST_ACCEL_GROUND : RL::BOOST_ACCEL_AIR) * UU_TO_BT * st_fwd(c) *
                                 RL::CAR_MASS_BT);
        s.time_since_boosted = 0;
    } else {
        s.time_since_boosted += dt;
    }
    s.boost = rs_min(s.boost, RL::BOOST_MAX);
}

void update_jump(Car& c, float dt, bool pressed) {  // Car::_UpdateJump (Car.cpp:535-582)
    rsg_car_state& s = c.st;
    if (s.is_on_ground && !s.is_jumping) {
        if (s.has_jumped && s.jump_time < RL::JUMP_MIN_TIME + RL::JUMP_RESET_TIME_PAD) {
        } else {
            s.has_jumped = 0;
            s.jump_time = 0;
        }
    }
    if (s.is_jumping) {
        s.is_jumping = (s.jump_time < RL::JUMP_MIN_TIME || (c.controls.jump && s.jump_time < RL::JUMP_MAX_TIME));
    } else if (s.is_on_ground && pressed) {
        s.is_jumping = 1;
        s.jump_time = 0;
        V3 f = st_up(c) * RL::JUMP_IMMEDIATE_FORCE * UU_TO_BT * RL::CAR_MASS_BT;
        c.rb.apply_central_impulse(f);
    }
    if (s.is_jumping) {
        s.has_jumped = 1;
        V3 tf = st_up(c) * RL::JUMP_ACCEL;
        if (s.jump_time < RL::JUMP_MIN_TIME) tf *= 0.62f;
        c.rb.apply_central_force(tf * UU_TO_BT * RL::CAR_MASS_BT);
    }
    if (s.is_jumping || s.has_jumped) s.jump_time += dt;
}

void update_air_torque(Car& c, float dt, bool update_air_control) {  // Car::_UpdateAirTorque (Car.cpp:584-669)
    rsg_car_state& s = c.st;
    V3 pitch_right = -st_right(c), yaw_up = st_up(c), roll_fwd = -st_fwd(c);
    bool do_air = false;
    if (s.is_flipping) s.is_flipping = s.has_flipped && s.flip_time < RL::FLIP_TORQUE_TIME;
    if (s.is_flipping) {
        V3 rel = V(s.flip_rel_torque);
        if (!is_zero(rel)) {
            float ps = 1;
            if (rel.y != 0 && c.controls.pitch != 0) {
                if (rs_sgn(rel.y) == rs_sgn(c.controls.pitch)) {
                    ps = 1 - rs_min(std::fabs(c.controls.pitch), 1);
                    do_air = true;
                }
            }
            rel.y *= ps;
            V3 dodge = rel * V3(RL::FLIP_TORQUE_X, RL::FLIP_TORQUE_Y, 0);
            c.rb.apply_torque(inverse(c.rb.inv_inertia_world) * c.rb.xf.b * dodge);
        } else {
            do_air = true;
        }
    } else {
        do_air = true;
    }
    do_air &= !s.is_auto_flipping;
    do_air &= update_air_control;
    if (do_air) {
        float pts = 1;
        V3 torque;
        if (c.controls.pitch || c.controls.yaw || c.controls.roll) {
            if (s.is_flipping) pts = 0;
            else if (s.has_flipped) {
                if (s.flip_time < RL::FLIP_TORQUE_TIME + RL::FLIP_PITCHLOCK_EXTRA_TIME) pts = 0;
            }
            torque = (c.controls.pitch * pitch_right * pts * RL::CAR_AIR_CONTROL_TORQUE.x) +
                     (c.controls.yaw * yaw_up * RL::CAR_AIR_CONTROL_TORQUE.y) +
                     (c.controls.roll * roll_fwd * RL::CAR_AIR_CONTROL_TORQUE.z);
        } else {
            torque = V3(0, 0, 0);
        }
        V3 av = c.rb.ang_vel;
        float dp = dot(pitch_right, av) * RL::CAR_AIR_CONTROL_DAMPING.x * (1 - std::fabs(do_air ? (c.controls.pitch * pts) : 0));
        float dy = dot(yaw_up, av) * RL::CAR_AIR_CONTROL_DAMPING.y * (1 - std::fabs(do_air ? c.controls.yaw : 0));
        float dr = dot(roll_fwd, av) * RL::CAR_AIR_CONTROL_DAMPING.z;
        V3 damping = (yaw_up * dy) + (pitch_right * dp) + (roll_fwd * dr);
        c.rb.apply_torque(inverse(c.rb.inv_inertia_world) * (torque - damping) * RL::CAR_TORQUE_SCALE);
    }
    if (c.controls.throttle != 0)
        c.rb.apply_central_force(st_fwd(c) * c.controls.throttle * RL::THROTTLE_AIR_ACCEL * UU_TO_BT * RL::CAR_MASS_BT);
}

void update_double_jump_or_flip(Car& c, float dt, bool pressed, float fwd_speed) {  // Car.cpp:671-781
    rsg_car_state& s = c.st;
    if (s.is_on_ground) {
        s.has_double_jumped = 0;
        s.has_flipped = 0;
        s.air_time = 0;
        s.air_time_since_jump = 0;
        s.flip_time = 0;
    } else {
        s.air_time += dt;
        if (s.has_jumped && !s.is_jumping) s.air_time_since_jump += dt;
        else s.air_time_since_jump = 0;
        if (pressed && s.air_time_since_jump < RL::DOUBLEJUMP_MAX_DELAY) {
            float mag = std::fabs(c.controls.yaw) + std::fabs(c.controls.pitch) + std::fabs(c.controls.roll);
            bool flip_input = mag >= c.cfg.dodge_deadzone;
            bool can = (!s.has_double_jumped && !s.has_flipped);
            if (s.is_auto_flipping) can = false;
            if (can) {
                if (flip_input) {
                    s.flip_time = 0;
                    s.has_flipped = 1;
                    s.is_flipping = 1;
                    float ratio = std::fabs(fwd_speed) / RL::CAR_MAX_SPEED;
                    V3 dd(-c.controls.pitch, c.controls.yaw + c.controls.roll, 0);
                    if (std::fabs(c.controls.yaw + c.controls.roll) < 0.1f && std::fabs(c.controls.pitch) < 0.1f) dd = V3(0, 0, 0);
                    else dd = safe_normalized(dd);
                    s.flip_rel_torque = P(V3(-dd.y, dd.x, 0));
                    if (std::fabs(dd.x) < 0.1f) dd.x = 0;
                    if (std::fabs(dd.y) < 0.1f) dd.y = 0;
                    if (!fuzzy_zero(dd)) {
                        bool back;
                        if (std::fabs(fwd_speed) < 100.0f) back = dd.x < 0.0f;
                        else back = (dd.x >= 0.0f) != (fwd_speed >= 0.0f);
                        V3 iv = dd * RL::FLIP_INITIAL_VEL_SCALE;
                        float msx = back ? RL::FLIP_BACKWARD_IMPULSE_MAX_SPEED_SCALE : RL::FLIP_FORWARD_IMPULSE_MAX_SPEED_SCALE;
                        iv.x *= ((msx - 1) * ratio) + 1.f;
                        iv.y *= ((RL::FLIP_SIDE_IMPULSE_MAX_SPEED_SCALE - 1) * ratio) + 1.f;
                        if (back) iv.x *= RL::FLIP_BACKWARD_IMPULSE_SCALE_X;
                        V3 f2 = st_fwd(c);
                        f2.z = 0;
                        f2 = rs_normalized(f2);
                        V3 r2(-f2.y, f2.x, 0.f);
                        V3 fdv = iv.x * f2 + iv.y * r2;
                        c.rb.apply_central_impulse(fdv * UU_TO_BT * RL::CAR_MASS_BT);
                    }
                } else {
                    V3 f = st_up(c) * RL::JUMP_IMMEDIATE_FORCE * UU_TO_BT * RL::CAR_MASS_BT;
                    c.rb.apply_central_impulse(f);
                    s.has_double_jumped = 1;
                }
            }
        }
    }
    if (s.is_flipping) {
        s.flip_time += dt;
        if (s.flip_time <= RL::FLIP_TORQUE_TIME) {
            if (s.flip_time >= RL::FLIP_Z_DAMP_START && (c.rb.lin_vel.z < 0 || s.flip_time < RL::FLIP_Z_DAMP_END))
                c.rb.lin_vel.z *= std::pow(1 - RL::FLIP_Z_DAMP_120, dt / (1 / 120.f));
        }
    } else if (s.has_flipped) {
        s.flip_time += dt;
    }
}

// Angle::FromRotMat (MathTypes.cpp:62-71) -> btMatrix3x3::getEulerYPR roll only
float roll_from_rot(const rsg_rotmat& r) {
    M3 m = rot_to_m3(r);
    float sp = -m.r[2].x;  // btAsin clamps to [-1, 1] (LinearMath/btScalar.h:510-516)
    sp = sp < -1.f ? -1.f : (sp > 1.f ? 1.f : sp);
    float pitch = std::asin(sp);
    float roll = std::atan2(m.r[2].y, m.r[2].z);
    if (std::fabs(pitch) == HALF_PI_F) {
        if (roll > 0) roll -= PI_F;
        else roll += PI_F;
    }
    return -roll;
}

void update_auto_flip(Car& c, float dt, bool pressed) {  // Car::_UpdateAutoFlip (Car.cpp:783-817)
    rsg_car_state& s = c.st;
    if (pressed && s.world_contact_has_contact && s.world_contact_normal.z > RL::CAR_AUTOFLIP_NORMZ_THRESH) {
        float roll = roll_from_rot(s.rot_mat);
        float ar = std::fabs(roll);
        if (ar > RL::CAR_AUTOFLIP_ROLL_THRESH) {
            s.auto_flip_timer = (float)(RL::CAR_AUTOFLIP_TIME * (ar / 3.14159265358979323846));
            s.auto_flip_torque_scale = (roll > 0) ? 1 : -1;
            s.is_auto_flipping = 1;
            c.rb.apply_central_impulse(-st_up(c) * RL::CAR_AUTOFLIP_IMPULSE * UU_TO_BT * RL::CAR_MASS_BT);
        }
    }
    if (s.is_auto_flipping) {
        if (s.auto_flip_timer <= 0) {
            s.is_auto_flipping = 0;
            s.auto_flip_timer = 0;
        } else {
            c.rb.ang_vel += st_fwd(c) * RL::CAR_AUTOFLIP_TORQUE * s.auto_flip_torque_scale * dt;
            s.auto_flip_timer -= dt;
        }
    }
}

void update_auto_roll(Car& c, int nwc) {  // Car::_UpdateAutoRoll (Car.cpp:819-853)
    rsg_car_state& s = c.st;
    V3 gup = nwc > 0 ? upwards_from_wheels(c) : V(s.world_contact_normal);
    V3 gdown = -gup;
    V3 f = st_fwd(c), r = st_right(c), u = st_up(c);
    V3 crossR = cross(gup, f), crossF = cross(gdown, crossR);
    float rtf = 1 - rs_clamp(dot(r, crossR), 0, 1);
    float ftf = 1 - rs_clamp(dot(f, crossF), 0, 1);
    V3 tdr = f * (dot(r, gup) >= 0 ? -1.f : 1.f);
    V3 tdf = r * (dot(f, gup) >= 0 ? 1.f : -1.f);
    V3 tr = tdr * rtf, tf = tdf * ftf;
    (void)u;
    c.rb.apply_central_force(gdown * RL::CAR_AUTOROLL_FORCE * UU_TO_BT * RL::CAR_MASS_BT);
    c.rb.apply_torque(inverse(c.rb.inv_inertia_world) * (tf + tr) * RL::CAR_AUTOROLL_TORQUE);
}

inline void clamp_controls(rsg_car_controls& k) {  // CarControls::ClampFix (CarControls.h:21-27)
    k.throttle = rs_clamp(k.throttle, -1, 1);
    k.steer = rs_clamp(k.steer, -1, 1);
    k.pitch = rs_clamp(k.pitch, -1, 1);
    k.yaw = rs_clamp(k.yaw, -1, 1);
    k.roll = rs_clamp(k.roll, -1, 1);
}

void car_pre_tick(Arena& a, Car& c) {  // Car::_PreTickUpdate (Car.cpp:58-131)
    float dt = a.tick_time;
    clamp_controls(c.controls);
    rsg_car_state& s = c.st;
    if (s.is_demoed) {
        s.demo_respawn_timer = rs_max(s.demo_respawn_timer - dt, 0);
        if (s.demo_respawn_timer == 0) car_respawn(c, 0, RL::BOOST_SPAWN_AMOUNT);
        c.rb.act = DISABLE_SIMULATION;
        c.rb.no_contact_response = true;
    } else {
        c.rb.act = ACTIVE_TAG;
        c.rb.no_contact_response = false;
    }
    if (s.is_demoed) return;
    for (int i = 0; i < 4; i++) update_wheel_transform(c, c.w[i]);
    for (int i = 0; i < 4; i++) ray_cast_wheel(a, c, c.w[i]);
    calc_friction_impulses(a, c, dt);
    bool pressed = c.controls.jump && !s.last_controls.jump;
    int nwc = 0;
    for (int i = 0; i < 4; i++) {
        bool ic = c.w[i].in_contact;
        s.wheels_with_contact[i] = ic;
        nwc += ic;
    }
    s.is_on_ground = nwc >= 3;
    float fwd_speed = dot(c.rb.lin_vel, chassis_fwd(c)) * BT_TO_UU;
    update_wheels(c, dt, nwc, fwd_speed);
    if (nwc < 3) update_air_torque(c, dt, nwc == 0);
    else s.is_flipping = 0;
    update_jump(c, dt, pressed);
    update_auto_flip(c, dt, pressed);
    update_double_jump_or_flip(c, dt, pressed, fwd_speed);
    if (c.controls.throttle && ((nwc > 0 && nwc < 4) || s.world_contact_has_contact)) update_auto_roll(c, nwc);
    s.world_contact_has_contact = 0;
    update_suspension(c, dt);
    apply_friction_impulses(c, dt);
    update_boost(c, dt);
}

void car_post_tick(Arena& a, Car& c) {  // Car::_PostTickUpdate (Car.cpp:133-163)
    rsg_car_state& s = c.st;
    if (s.is_demoed) return;
    s.rot_mat = m3_to_rot(c.rb.xf.b);
    float sp2 = len2(c.rb.lin_vel * BT_TO_UU);
    if (s.is_supersonic && s.supersonic_time < RL::SUPERSONIC_MAINTAIN_MAX_TIME)
        s.is_supersonic = (sp2 >= RL::SUPERSONIC_MAINTAIN_MIN_SPEED * RL::SUPERSONIC_MAINTAIN_MIN_SPEED);
    else
        s.is_supersonic = (sp2 >= RL::SUPERSONIC_START_SPEED * RL::SUPERSONIC_START_SPEED);
    if (s.is_supersonic) s.supersonic_time += a.tick_time;
    else s.supersonic_time = 0;
    if (s.car_contact_cooldown_timer > 0)
        s.car_contact_cooldown_timer = rs_max(s.car_contact_cooldown_timer - a.tick_time, 0);
    s.last_controls = c.controls;
}

void car_finish_physics(Car& c) {  // Car::_FinishPhysicsTick (Car.cpp:165-193)
    rsg_car_state& s = c.st;
    if (s.is_demoed) return;
    if (!is_zero(c.vel_impulse_cache)) {
        c.rb.lin_vel += c.vel_impulse_cache;
        c.vel_impulse_cache = V3(0, 0, 0);
    }
    V3 v = c.rb.lin_vel, w = c.rb.ang_vel;
    if (len2(v) > (RL::CAR_MAX_SPEED * UU_TO_BT) * (RL::CAR_MAX_SPEED * UU_TO_BT)) v = normalized(v) * (RL::CAR_MAX_SPEED * UU_TO_BT);
    if (len2(w) > (RL::CAR_MAX_ANG_SPEED * RL::CAR_MAX_ANG_SPEED)) w = normalized(w) * RL::CAR_MAX_ANG_SPEED;
    c.rb.lin_vel = v;
    c.rb.ang_vel = w;
    s.tick_count_since_update++;
}

// ================================================================ shapes / AABBs
void car_child_xf(const Car& c, Xf& out) {  // compound child: car transform * hitbox offset
    Xf off = xf_identity();
    off.o = c.hitbox_off;
    out = xf_mul(c.rb.xf, off);
}
void car_box_aabb(const Car& c, const Xf& child, V3& mn, V3& mx) {
    transform_aabb(c.hitbox_he, c.hitbox_margin, child, mn, mx);
}
void car_compound_aabb(const Car& c, const Xf& t, V3& mn, V3& mx) {  // btCompoundShape::getAabb
    V3 lhe = 0.5f * (c.comp_max - c.comp_min);
    V3 lc = 0.5f * (c.comp_max + c.comp_min);
    M3 ab = absolute(t.b);
    V3 center = xf_apply(t, lc);
    V3 ext(dot(ab.r[0], lhe), dot(ab.r[1], lhe), dot(ab.r[2], lhe));
    mn = center - ext;
    mx = center + ext;
}
void ball_aabb(const Arena& a, const Xf& t, V3& mn, V3& mx) {
    float m = a.ball_radius + 0.08f;
    mn = t.o - V3(m, m, m);
    mx = t.o + V3(m, m, m);
}
void mesh_aabb(V3& mn, V3& mx) {  // btTriangleMeshShape::getAabb with identity
    const Mesh& m = *g_mesh;
    V3 lhe = 0.5f * (m.aabb_max - m.aabb_min);
    V3 lc = 0.5f * (m.aabb_max + m.aabb_min);
    mn = lc - lhe;
    mx = lc + lhe;
}

// btTransformUtil::integrateTransform (B/LinearMath/btTransformUtil.h:37-80)
void integrate_transform(const Xf& cur, V3 lv, V3 av, float dt, bool no_rot, Xf& out) {
    out.o = cur.o + lv * dt;
    if (no_rot) { out.b = cur.b; return; }
    const float ANGULAR_MOTION_THRESHOLD = 0.5f * HALF_PI_F;
    float a2 = len2(av);
    float ang = 0;
    if (a2 > SIMD_EPS) ang = std::sqrt(a2);
    if (ang * dt > ANGULAR_MOTION_THRESHOLD) ang = ANGULAR_MOTION_THRESHOLD / dt;
    V3 axis;
    if (ang < 0.001f) axis = av * (0.5f * dt - (dt * dt * dt) * (0.020833333333f) * ang * ang);
    else axis = av * (std::sin(0.5f * ang * dt) / ang);
    Q dorn(axis.x, axis.y, axis.z, std::cos(ang * dt * 0.5f));
    Q orn0 = q_from_m(cur.b);
    Q pred = q_mul(dorn, orn0);
    pred = q_safe_normalize(pred);
    if (q_len2(pred) > SIMD_EPS) out.b = m_from_q(pred);
    else out.b = cur.b;
}

// ================================================================ narrow phase
struct Contact {  // what a detector hands to btManifoldResult::addContactPoint
    V3 normal_on_b, point_on_b;
    float depth;
};

// btManifoldResult::addContactPoint (B/.../CollisionDispatch/btManifoldResult.cpp:109-194):
// adds into manifold `m`; `swapped` tells that the detector's (A,B) are (body1,body0) of m
int add_point(Arena& a, Manifold& m, const Xf& x0, const Xf& x1, V3 n, V3 pb, float depth, bool swapped,
              float friction, float restitution) {
    if (depth > m.breaking) return -1;
    V3 pa = pb + n * depth;
    MPoint p;
    if (swapped) {
        p.local_a = xf_inv_apply(x0, pa);  // manifold body0 is the detector's B object
        p.local_b = xf_inv_apply(x1, pb);
    } else {
        p.local_a = xf_inv_apply(x0, pa);
        p.local_b = xf_inv_apply(x1, pb);
    }
    p.normal = n;
    p.dist = depth;
    p.pos_a = pa;
    p.pos_b = pb;
    p.friction = friction;
    p.restitution = restitution;
    int idx;
    if (m.n == 4) {
        // btPersistentManifold::sortCachedPoints (btPersistentManifold.cpp:113-190)
        int maxPen = -1;
        float maxv = p.dist;
        for (int i = 0; i < 4; i++)
            if (m.pts[i].dist < maxv) { maxPen = i; maxv = m.pts[i].dist; }
        float r0 = 0, r1 = 0, r2 = 0, r3 = 0;
        if (maxPen != 0) r0 = len2(cross(p.local_a - m.pts[1].local_a, m.pts[3].local_a - m.pts[2].local_a));
        if (maxPen != 1) r1 = len2(cross(p.local_a - m.pts[0].local_a, m.pts[3].local_a - m.pts[2].local_a));
        if (maxPen != 2) r2 = len2(cross(p.local_a - m.pts[0].local_a, m.pts[3].local_a - m.pts[1].local_a));
        if (maxPen != 3) r3 = len2(cross(p.local_a - m.pts[0].local_a, m.pts[2].local_a - m.pts[1].local_a));
        idx = closest_axis4(r0, r1, r2, r3);
        if (idx < 0) idx = 0;
    } else {
        idx = m.n++;
    }
    m.pts[idx] = p;
    a.counters[0]++;
    return idx;
}

// btPersistentManifold::refreshContactPoints (btPersistentManifold.cpp:263-318)
void refresh(Manifold& m, const Xf& x0, const Xf& x1) {
    for (int i = m.n - 1; i >= 0; i--) {
        MPoint& p = m.pts[i];
        p.pos_a = xf_apply(x0, p.local_a);
        p.pos_b = xf_apply(x1, p.local_b);
        p.dist = dot(p.pos_a - p.pos_b, p.normal);
    }
    for (int i = m.n - 1; i >= 0; i--) {
        MPoint& p = m.pts[i];
        bool remove = false;
        if (!(p.dist <= m.breaking)) remove = true;
        else {
            V3 proj = p.pos_a - p.normal * p.dist;
            V3 diff = p.pos_b - proj;
            if (dot(diff, diff) > m.breaking * m.breaking) remove = true;
        }
        if (remove) {
            int last = m.n - 1;
            if (i != last) m.pts[i] = m.pts[last];
            m.n--;
        }
    }
}

// btAdjustInternalEdgeContacts (btInternalEdgeUtility.cpp:414-840) for a mesh triangle
// contact; mesh transform is identity.  Flags argument of the reference call is 0.
void nearest_on_segment(V3 p, V3 l0, V3 l1, V3& out) {
    V3 d = l1 - l0;
    if (fuzzy_zero(d)) { out = l0; return; }
    float t = dot(p - l0, d) / dot(d, d);
    if (t < 0) t = 0;
    else if (t > 1) t = 1;
    out = l0 + d * t;
}
bool clamp_normal(V3 edge, V3 tri_n, V3 local_n, float corrected, V3& out) {
    V3 ec = normalized(cross(edge, tri_n));
    float cur = std::atan2(dot(local_n, ec), dot(local_n, tri_n));
    if (corrected < 0) {
        if (cur < corrected) {
            Q rot = q_axis_angle(edge, corrected - cur);
            out = m_from_q(rot) * local_n;
            return true;
        }
    }
    if (corrected >= 0) {
        if (cur > corrected) {
            Q rot = q_axis_angle(edge, corrected - cur);
            out = m_from_q(rot) * local_n;
            return true;
        }
    }
    return false;
}
void adjust_internal_edge(MPoint& cp, int tri) {
    const Mesh& m = *g_mesh;
    const TriInfo& inf = m.info[tri];
    if (!inf.present) return;
    V3 v[3];
    m.tri_verts(tri, v);
    V3 tri_n = normalized(cross(v[1] - v[0], v[2] - v[0]));
    V3 nearest;
    nearest_on_segment(cp.local_b, v[0], v[1], nearest);
    V3 contact = cp.local_b;
    bool near_edge = false;
    int concave = 0;
    V3 lcn = normalized(cp.normal);  // basis is identity
    int best = -1;
    float bestd = BT_LARGE;
    const float MAXA = TWO_PI_F, EDGE_D = 0.1f, CONVEX_EPS = 0.f;
    if (std::fabs(inf.a01) < MAXA) {
        V3 nn; nearest_on_segment(cp.local_b, v[0], v[1], nn);
        float l = len(contact - nn);
        if (l < bestd) { best = 0; bestd = l; }
    }
    if (std::fabs(inf.a12) < MAXA) {
        V3 nn; nearest_on_segment(cp.local_b, v[1], v[2], nn);
        float l = len(contact - nn);
        if (l < bestd) { best = 1; bestd = l; }
    }
    if (std::fabs(inf.a20) < MAXA) {
        V3 nn; nearest_on_segment(cp.local_b, v[2], v[0], nn);
        float l = len(contact - nn);
        if (l < bestd) { best = 2; bestd = l; }
    }
    auto edge_case = [&](int which, V3 edge, float angle, int convflag, int swapflag, bool recompute_local) {
        near_edge = true;
        if (angle == 0.f) { concave++; return; }
        bool conv = (inf.flags & convflag) != 0;
        float sf = conv ? 1.f : -1.f;
        V3 nA = sf * tri_n;
        Q orn = q_axis_angle(edge, angle);
        V3 cnB = q_rotate(orn, tri_n);
        if (inf.flags & swapflag) cnB *= -1;
        V3 nB = sf * cnB;
        float ndA = dot(lcn, nA), ndB = dot(lcn, nB);
        bool back = (ndA < CONVEX_EPS) && (ndB < CONVEX_EPS);
        if (back) { concave++; return; }
        V3 ln = recompute_local ? cp.normal : lcn;
        V3 clamped;
        if (clamp_normal(edge, sf * tri_n, ln, angle, clamped)) {
            if (dot(clamped, tri_n) > 0) {
                cp.normal = clamped;
                cp.pos_b = cp.pos_a - cp.normal * cp.dist;
                cp.local_b = cp.pos_b;
            }
        }
        (void)which;
    };
    if (std::fabs(inf.a01) < MAXA) {
        float l = len(contact - nearest);
        if (l < EDGE_D && best == 0) edge_case(0, v[0] - v[1], inf.a01, TRI_V0V1_CONVEX, TRI_V0V1_SWAP, false);
    }
    nearest_on_segment(contact, v[1], v[2], nearest);
    if (std::fabs(inf.a12) < MAXA) {
        float l = len(contact - nearest);
        if (l < EDGE_D && best == 1) edge_case(1, v[1] - v[2], inf.a12, TRI_V1V2_CONVEX, TRI_V1V2_SWAP, true);
    }
    nearest_on_segment(contact, v[2], v[0], nearest);
    if (std::fabs(inf.a20) < MAXA) {
        float l = len(contact - nearest);
        if (l < EDGE_D && best == 2) edge_case(2, v[2] - v[0], inf.a20, TRI_V2V0_CONVEX, TRI_V2V0_SWAP, true);
    }
    if (near_edge && concave > 0) {
        V3 nn = tri_n;
        float d = dot(nn, lcn);
        if (d < 0) return;
        cp.normal = nn;
        cp.pos_b = cp.pos_a - cp.normal * cp.dist;
        cp.local_b = cp.pos_b;
    }
}

// ---------------------------------------------------------------- GJK
// btGjkPairDetector::getClosestPointsNonVirtual (btGjkPairDetector.cpp:693-959) with
// btVoronoiSimplexSolver (btVoronoiSimplexSolver.cpp), restated.
struct Convex {
    int type;  // 0 box (half extents he), 1 sphere (point core), 2 triangle
    V3 he;
    V3 tv[3];
    float margin;
    V3 support_nomargin(V3 d) const {
        if (type == 0) return V3(d.x >= 0 ? he.x : -he.x, d.y >= 0 ? he.y : -he.y, d.z >= 0 ? he.z : -he.z);
        if (type == 1) return V3(0, 0, 0);
        V3 dots(dot(d, tv[0]), dot(d, tv[1]), dot(d, tv[2]));
        return tv[max_axis(dots)];
    }
    void aabb(const Xf& t, V3& mn, V3& mx) const {  // used by m_fixContactNormalDirection
        if (type == 0) { transform_aabb(he, margin, t, mn, mx); return; }
        if (type == 1) {
            float m = margin + 0.08f;
            mn = t.o - V3(m, m, m);
            mx = t.o + V3(m, m, m);
            return;
        }
        // btTriangleShape::getAabb -> btPolyhedralConvexAabbCachingShape... uses support in 6 dirs
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
    bool used[4] = {false, false, false, false};
    float bary[4] = {0, 0, 0, 0};
    bool degenerate = false;
    void reset() {
        degenerate = false;
        for (int i = 0; i < 4; i++) { used[i] = false; bary[i] = 0; }
    }
    bool valid() const { return bary[0] >= 0 && bary[1] >= 0 && bary[2] >= 0 && bary[3] >= 0; }
    void set_bary(float a, float b, float c, float d) { bary[0] = a; bary[1] = b; bary[2] = c; bary[3] = d; }
};

struct Simplex {
    int n = 0;
    V3 W[5], Pp[5], Qq[5];
    V3 lastW;
    bool needs_update = true, cached_valid = false;
    V3 cP1, cP2, cV;
    SubResult bc;
    void reset() {
        cached_valid = false;
        n = 0;
        needs_update = true;
        lastW = V3(BT_LARGE, BT_LARGE, BT_LARGE);
        bc.reset();
    }
    void remove(int i) {
        n--;
        W[i] = W[n]; Pp[i] = Pp[n]; Qq[i] = Qq[n];
    }
    void reduce(const SubResult& r) {
        if (n >= 4 && !r.used[3]) remove(3);
        if (n >= 3 && !r.used[2]) remove(2);
        if (n >= 2 && !r.used[1]) remove(1);
        if (n >= 1 && !r.used[0]) remove(0);
    }
    void add(V3 w, V3 p, V3 q) {
        lastW = w;
        needs_update = true;
        W[n] = w; Pp[n] = p; Qq[n] = q;
        n++;
    }
    static bool closest_tri(V3 p, V3 a, V3 b, V3 c, SubResult& r) {
        r.used[0] = r.used[1] = r.used[2] = r.used[3] = false;
        V3 ab = b - a, ac = c - a, ap = p - a;
        float d1 = dot(ab, ap), d2 = dot(ac, ap);
        if (d1 <= 0.f && d2 <= 0.f) { r.closest = a; r.used[0] = true; r.set_bary(1, 0, 0, 0); return true; }
        V3 bp = p - b;
        float d3 = dot(ab, bp), d4 = dot(ac, bp);
        if (d3 >= 0.f && d4 <= d3) { r.closest = b; r.used[1] = true; r.set_bary(0, 1, 0, 0); return true; }
        float vc = d1 * d4 - d3 * d2;
        if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
            float v = d1 / (d1 - d3);
            r.closest = a + v * ab; r.used[0] = r.used[1] = true; r.set_bary(1 - v, v, 0, 0);
            return true;
        }
        V3 cp = p - c;
        float d5 = dot(ab, cp), d6 = dot(ac, cp);
        if (d6 >= 0.f && d5 <= d6) { r.closest = c; r.used[2] = true; r.set_bary(0, 0, 1, 0); return true; }
        float vb = d5 * d2 - d1 * d6;
        if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
            float w = d2 / (d2 - d6);
            r.closest = a + w * ac; r.used[0] = r.used[2] = true; r.set_bary(1 - w, 0, w, 0);
            return true;
        }
        float va = d3 * d6 - d5 * d4;
        if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
            float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            r.closest = b + w * (c - b); r.used[1] = r.used[2] = true; r.set_bary(0, 1 - w, w, 0);
            return true;
        }
        float denom = 1.f / (va + vb + vc);
        float v = vb * denom, w = vc * denom;
        r.closest = a + ab * v + ac * w;
        r.used[0] = r.used[1] = r.used[2] = true;
        r.set_bary(1 - v - w, v, w, 0);
        return true;
    }
    static int outside(V3 p, V3 a, V3 b, V3 c, V3 d) {
        V3 nrm = cross(b - a, c - a);
        float sp = dot(p - a, nrm), sd = dot(d - a, nrm);
        if (sd * sd < (1e-4f * 1e-4f)) return -1;
        return sp * sd < 0.f;
    }
    static bool closest_tet(V3 p, V3 a, V3 b, V3 c, V3 d, SubResult& fr) {
        SubResult t;
        fr.closest = p;
        fr.used[0] = fr.used[1] = fr.used[2] = fr.used[3] = true;
        int oABC = outside(p, a, b, c, d), oACD = outside(p, a, c, d, b), oADB = outside(p, a, d, b, c),
            oBDC = outside(p, b, d, c, a);
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
    bool update() {
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
    bool closest(V3& v) { bool ok = update(); v = cV; return ok; }
    bool in_simplex(V3 w) const {
        bool found = false;
        for (int i = 0; i < n; i++)
            if (len2(W[i] - w) <= 0.0001f) { found = true; break; }
        if (w == lastW) return true;
        return found;
    }
    void points(V3& p1, V3& p2) { update(); p1 = cP1; p2 = cP2; }
};

// btSubsimplexConvexCast::calcTimeOfImpact (B/BulletCollision/NarrowPhaseCollision/btSubSimplexConvexCast.cpp:30-141)
// of a point (btSphereShape of radius and margin 0, btCollisionWorld.cpp:271-273) moving from `from`
// to `to` against a static convex shape whose world support vertex for a world direction d is
// `support(d, o)` with the shape's origin at o; then the acceptance of
// btCollisionWorld::rayTestSingleInternal (btCollisionWorld.cpp:288-310): a normal longer than 0.01
// and a fraction below the closest hit so far.  The shape's transform is interpolated like the
// point's (btSubSimplexConvexCast.cpp:93-94), between two equal origins, which moves it by rounding.
// MAX_CONVEX_CAST_ITERATIONS 32, MAX_CONVEX_CAST_EPSILON 1e-4 (btConvexCast.h:28-29), no allowed
// penetration; the point's supporting vertex is its origin.
template <class Sup>
bool ray_subsimplex(V3 from, V3 to, V3 ob, Sup support, float& hit_frac, V3& out_normal) {
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
    out_normal = normalized(nrm);
    return true;
}

// btBoxShape::localGetSupportingVertex (btBoxShape.h:47-56), half extents with the margin
bool ray_cast_box(V3 from, V3 to, const Xf& box_xf, V3 he_margin, float& hit_frac, V3& out_normal) {
    auto sup = [&](V3 d, V3 o) {
        V3 l = transpose(box_xf.b) * d;  // d * basis
        V3 s(l.x >= 0.f ? he_margin.x : -he_margin.x, l.y >= 0.f ? he_margin.y : -he_margin.y,
             l.z >= 0.f ? he_margin.z : -he_margin.z);
        Xf t = box_xf;
        t.o = o;
        return xf_apply(t, s);
    };
    return ray_subsimplex(from, to, box_xf.o, sup, hit_frac, out_normal);
}

// btSphereShape::localGetSupportingVertex (btSphereShape.cpp:37-49): the margin (the radius) along the
// normalised direction, (-1,-1,-1) normalised for a vanishing one
bool ray_cast_sphere(V3 from, V3 to, const Xf& xf, float radius, float& hit_frac, V3& out_normal) {
    auto sup = [&](V3 d, V3 o) {
        V3 l = transpose(xf.b) * d;
        if (len2(l) < (SIMD_EPS * SIMD_EPS)) l = normalized(V3(-1, -1, -1));
        else l = normalized(l);
        Xf t = xf;
        t.o = o;
        return xf_apply(t, l * radius);
    };
    return ray_subsimplex(from, to, xf.o, sup, hit_frac, out_normal);
}

// ---------------------------------------------------------------- GJK + EPA penetration depth
// btGjkEpa2 (B/BulletCollision/NarrowPhaseCollision/btGjkEpa2.cpp) as btGjkEpaPenetrationDepthSolver
// (btGjkEpaPenetrationDepthSolver.cpp:22-77) drives it: everything is expressed in shape A's
// frame, supports include the margins, and the polytope lives in fixed pools linked by index.
namespace epa {
constexpr int GJK_MAX_ITER = 128;
constexpr float GJK_ACCURACY = 0.0001f, GJK_MIN_DISTANCE = 0.0001f, GJK_DUPLICATED_EPS = 0.0001f;
constexpr int EPA_MAX_VERTICES = 128, EPA_MAX_FACES = 256, EPA_MAX_ITER = 255;
constexpr float EPA_ACCURACY = 0.0001f, EPA_PLANE_EPS = 0.00001f;

// btConvexShape::localGetSupportVertexNonVirtual (btConvexShape.cpp:183-193)
inline V3 support_margin(const Convex& c, V3 d) {
    V3 n = d;
    if (len2(n) < SIMD_EPS * SIMD_EPS) n = V3(-1, -1, -1);
    n = normalized(n);
    return c.support_nomargin(n) + c.margin * n;
}

struct Minkowski {  // MinkowskiDiff (btGjkEpa2.cpp:80-150) with margins
    const Convex* a;
    const Convex* b;
    M3 to_b;   // m_toshape1: A-frame direction -> B frame
    Xf b_to_a; // m_toshape0: B-frame point -> A frame
    bool margins;
    V3 sup_a(V3 d) const { return margins ? support_margin(*a, d) : a->support_nomargin(d); }
    V3 sup_b(V3 d) const {
        V3 db = to_b * d;
        return xf_apply(b_to_a, margins ? support_margin(*b, db) : b->support_nomargin(db));
    }
    V3 sup(V3 d) const { return sup_a(d) - sup_b(-d); }
    V3 sup(V3 d, int which) const { return which ? sup_b(d) : sup_a(d); }
};

struct SV { V3 d, w; };
struct Simplex { int c[4]; float p[4]; int rank; };

// GJK of btGjkEpa2 (btGjkEpa2.cpp:155-581); support vertices live in sv[] (4 for GJK, the rest
// for EPA), the free list in freel[].
struct Solver {
    Minkowski shape;
    SV sv[4 + EPA_MAX_VERTICES];
    int freel[4], nfree;
    Simplex sims[2];
    int cur;
    V3 ray;
    int status;  // 0 valid, 1 inside, 2 failed
    Simplex* simplex;

    void getsupport(V3 d, SV& s) const {
        s.d = d / len(d);
        s.w = shape.sup(s.d);
    }
    void remove_vertex(Simplex& sx) { freel[nfree++] = sx.c[--sx.rank]; }
    void append_vertex(Simplex& sx, V3 v) {
        sx.p[sx.rank] = 0;
        sx.c[sx.rank] = freel[--nfree];
        getsupport(v, sv[sx.c[sx.rank++]]);
    }
    static float det(V3 a, V3 b, V3 c) {
        return (a.y * b.z * c.x + a.z * b.x * c.y - a.x * b.z * c.y - a.y * b.x * c.z + a.x * b.y * c.z -
                a.z * b.y * c.x);
    }
    static float project2(V3 a, V3 b, float* w, unsigned& m) {
        V3 d = b - a;
        float l = len2(d);
        if (l > 0.f) {
            float t = (l > 0 ? -dot(a, d) / l : 0);
            if (t >= 1) { w[0] = 0; w[1] = 1; m = 2; return len2(b); }
            if (t <= 0) { w[0] = 1; w[1] = 0; m = 1; return len2(a); }
            w[0] = 1 - (w[1] = t);
            m = 3;
            return len2(a + d * t);
        }
        return -1;
    }
    static float project3(V3 a, V3 b, V3 c, float* w, unsigned& m) {
        static const int imd3[] = {1, 2, 0};
        const V3* vt[] = {&a, &b, &c};
        const V3 dl[] = {a - b, b - c, c - a};
        const V3 n = cross(dl[0], dl[1]);
        const float l = len2(n);
        if (l > 0.f) {
            float mindist = -1;
            float subw[2] = {0.f, 0.f};
            unsigned subm = 0;
            for (int i = 0; i < 3; ++i) {
                if (dot(*vt[i], cross(dl[i], n)) > 0) {
                    const int j = imd3[i];
                    const float subd = project2(*vt[i], *vt[j], subw, subm);
                    if ((mindist < 0) || (subd < mindist)) {
                        mindist = subd;
                        m = ((subm & 1) ? 1u << i : 0) + ((subm & 2) ? 1u << j : 0);
                        w[i] = subw[0];
                        w[j] = subw[1];
                        w[imd3[j]] = 0;
                    }
                }
            }
            if (mindist < 0) {
                const float d = dot(a, n);
                const float s = std::sqrt(l);
                const V3 p = n * (d / l);
                mindist = len2(p);
                m = 7;
                w[0] = len(cross(dl[1], b - p)) / s;
                w[1] = len(cross(dl[2], c - p)) / s;
                w[2] = 1 - (w[0] + w[1]);
            }
            return mindist;
        }
        return -1;
    }
    static float project4(V3 a, V3 b, V3 c, V3 d, float* w, unsigned& m) {
        static const int imd3[] = {1, 2, 0};
        const V3* vt[] = {&a, &b, &c, &d};
        const V3 dl[] = {a - d, b - d, c - d};
        const float vl = det(dl[0], dl[1], dl[2]);
        const bool ng = (vl * dot(a, cross(b - c, a - b))) <= 0;
        if (ng && (std::fabs(vl) > 0.f)) {
            float mindist = -1;
            float subw[3] = {0.f, 0.f, 0.f};
            unsigned subm = 0;
            for (int i = 0; i < 3; ++i) {
                const int j = imd3[i];
                const float s = vl * dot(d, cross(dl[i], dl[j]));
                if (s > 0) {
                    const float subd = project3(*vt[i], *vt[j], d, subw, subm);
                    if ((mindist < 0) || (subd < mindist)) {
                        mindist = subd;
                        m = (subm & 1 ? 1u << i : 0) + (subm & 2 ? 1u << j : 0) + (subm & 4 ? 8 : 0);
                        w[i] = subw[0];
                        w[j] = subw[1];
                        w[imd3[j]] = 0;
                        w[3] = subw[2];
                    }
                }
            }
            if (mindist < 0) {
                mindist = 0;
                m = 15;
                w[0] = det(c, b, d) / vl;
                w[1] = det(a, c, d) / vl;
                w[2] = det(b, a, d) / vl;
                w[3] = 1 - (w[0] + w[1] + w[2]);
            }
            return mindist;
        }
        return -1;
    }
    // GJK::Evaluate (btGjkEpa2.cpp:196-324)
    int evaluate(V3 guess) {
        int iterations = 0;
        float sqdist = 0, alpha = 0;
        V3 lastw[4];
        int clastw = 0;
        for (int i = 0; i < 4; i++) freel[i] = i;
        nfree = 4;
        cur = 0;
        status = 0;
        sims[0].rank = 0;
        ray = guess;
        const float sqrl = len2(ray);
        append_vertex(sims[0], sqrl > 0 ? -ray : V3(1, 0, 0));
        sims[0].p[0] = 1;
        ray = sv[sims[0].c[0]].w;
        sqdist = sqrl;
        lastw[0] = lastw[1] = lastw[2] = lastw[3] = ray;
        do {
            const int next = 1 - cur;
            Simplex& cs = sims[cur];
            Simplex& ns = sims[next];
            const float rl = len(ray);
            if (rl < GJK_MIN_DISTANCE) { status = 1; break; }
            append_vertex(cs, -ray);
            const V3 w = sv[cs.c[cs.rank - 1]].w;
            bool found = false;
            for (int i = 0; i < 4; ++i)
                if (len2(w - lastw[i]) < GJK_DUPLICATED_EPS) { found = true; break; }
            if (found) { remove_vertex(sims[cur]); break; }
            lastw[clastw = (clastw + 1) & 3] = w;
            const float omega = dot(ray, w) / rl;
            alpha = omega > alpha ? omega : alpha;
            if (((rl - alpha) - (GJK_ACCURACY * rl)) <= 0) { remove_vertex(sims[cur]); break; }
            float weights[4];
            unsigned mask = 0;
            switch (cs.rank) {
                case 2: sqdist = project2(sv[cs.c[0]].w, sv[cs.c[1]].w, weights, mask); break;
                case 3: sqdist = project3(sv[cs.c[0]].w, sv[cs.c[1]].w, sv[cs.c[2]].w, weights, mask); break;
                case 4:
                    sqdist = project4(sv[cs.c[0]].w, sv[cs.c[1]].w, sv[cs.c[2]].w, sv[cs.c[3]].w, weights, mask);
                    break;
            }
            if (sqdist >= 0) {
                ns.rank = 0;
                ray = V3(0, 0, 0);
                cur = next;
                for (int i = 0, ni = cs.rank; i < ni; ++i) {
                    if (mask & (1u << i)) {
                        ns.c[ns.rank] = cs.c[i];
                        ns.p[ns.rank++] = weights[i];
                        ray += sv[cs.c[i]].w * weights[i];
                    } else {
                        freel[nfree++] = cs.c[i];
                    }
                }
                if (mask == 15) status = 1;
            } else {
                remove_vertex(sims[cur]);
                break;
            }
            status = ((++iterations) < GJK_MAX_ITER) ? status : 2;
        } while (status == 0);
        simplex = &sims[cur];
        return status;
    }
    // GJK::EncloseOrigin (btGjkEpa2.cpp:325-389), its recursion unrolled by simplex rank
    bool enclose4() {
        return std::fabs(det(sv[simplex->c[0]].w - sv[simplex->c[3]].w, sv[simplex->c[1]].w - sv[simplex->c[3]].w,
                             sv[simplex->c[2]].w - sv[simplex->c[3]].w)) > 0;
    }
    bool enclose3() {
        const V3 n = cross(sv[simplex->c[1]].w - sv[simplex->c[0]].w, sv[simplex->c[2]].w - sv[simplex->c[0]].w);
        if (len2(n) > 0) {
            append_vertex(*simplex, n);
            if (enclose4()) return true;
            remove_vertex(*simplex);
            append_vertex(*simplex, -n);
            if (enclose4()) return true;
            remove_vertex(*simplex);
        }
        return false;
    }
    bool enclose2() {
        const V3 d = sv[simplex->c[1]].w - sv[simplex->c[0]].w;
        for (int i = 0; i < 3; ++i) {
            V3 axis(0, 0, 0);
            axis[i] = 1;
            const V3 p = cross(d, axis);
            if (len2(p) > 0) {
                append_vertex(*simplex, p);
                if (enclose3()) return true;
                remove_vertex(*simplex);
                append_vertex(*simplex, -p);
                if (enclose3()) return true;
                remove_vertex(*simplex);
            }
        }
        return false;
    }
    bool enclose1() {
        for (int i = 0; i < 3; ++i) {
            V3 axis(0, 0, 0);
            axis[i] = 1;
            append_vertex(*simplex, axis);
            if (enclose2()) return true;
            remove_vertex(*simplex);
            append_vertex(*simplex, -axis);
            if (enclose2()) return true;
            remove_vertex(*simplex);
        }
        return false;
    }
    bool enclose_origin() {
        switch (simplex->rank) {
            case 1: return enclose1();
            case 2: return enclose2();
            case 3: return enclose3();
            case 4: return enclose4();
        }
        return false;
    }
};

// EPA (btGjkEpa2.cpp:583-950): faces in a pool, hull and stock as doubly linked lists by index
struct Face {
    V3 n;
    float d;
    int c[3];     // support vertices (indices into Solver::sv)
    int f[3];     // neighbour faces
    int l[2];     // list links
    uint8_t e[3]; // neighbour edges
    uint8_t pass;
};
struct List { int root = -1; int count = 0; };

struct Epa {
    Face fc[EPA_MAX_FACES];
    List hull, stock;
    int nextsv;  // next free EPA support vertex (Solver::sv[4 + nextsv])
    int status;  // 0 valid, ..., see eStatus; only Failed (9) matters to the caller
    V3 normal;
    float depth;
    Simplex result;

    void bind(int fa, int ea, int fb, int eb) {
        fc[fa].e[ea] = (uint8_t)eb;
        fc[fa].f[ea] = fb;
        fc[fb].e[eb] = (uint8_t)ea;
        fc[fb].f[eb] = fa;
    }
    void append(List& list, int face) {
        fc[face].l[0] = -1;
        fc[face].l[1] = list.root;
        if (list.root >= 0) fc[list.root].l[0] = face;
        list.root = face;
        ++list.count;
    }
    void remove(List& list, int face) {
        if (fc[face].l[1] >= 0) fc[fc[face].l[1]].l[0] = fc[face].l[0];
        if (fc[face].l[0] >= 0) fc[fc[face].l[0]].l[1] = fc[face].l[1];
        if (face == list.root) list.root = fc[face].l[1];
        --list.count;
    }
    void init() {
        status = 9;
        normal = V3(0, 0, 0);
        depth = 0;
        nextsv = 0;
        hull = List();
        stock = List();
        for (int i = 0; i < EPA_MAX_FACES; ++i) append(stock, EPA_MAX_FACES - i - 1);
    }
    bool edge_dist(const Solver& g, int face, int a, int b, float& dist) {
        const V3 aw = g.sv[a].w, bw = g.sv[b].w;
        const V3 ba = bw - aw;
        const V3 n_ab = cross(ba, fc[face].n);
        const float a_dot_nab = dot(aw, n_ab);
        if (a_dot_nab < 0) {
            const float ba_l2 = len2(ba);
            const float a_dot_ba = dot(aw, ba);
            const float b_dot_ba = dot(bw, ba);
            if (a_dot_ba > 0) dist = len(aw);
            else if (b_dot_ba < 0) dist = len(bw);
            else {
                const float a_dot_b = dot(aw, bw);
                float v = (len2(aw) * len2(bw) - a_dot_b * a_dot_b) / ba_l2;
                dist = std::sqrt(v > 0.f ? v : 0.f);
            }
            return true;
        }
        return false;
    }
    int newface(const Solver& g, int a, int b, int c, bool forced) {
        if (stock.root >= 0) {
            int face = stock.root;
            remove(stock, face);
            append(hull, face);
            Face& F = fc[face];
            F.pass = 0;
            F.c[0] = a;
            F.c[1] = b;
            F.c[2] = c;
            F.n = cross(g.sv[b].w - g.sv[a].w, g.sv[c].w - g.sv[a].w);
            const float l = len(F.n);
            const bool v = l > EPA_ACCURACY;
            if (v) {
                if (!(edge_dist(g, face, a, b, F.d) || edge_dist(g, face, b, c, F.d) ||
                      edge_dist(g, face, c, a, F.d)))
                    F.d = dot(g.sv[a].w, F.n) / l;
                F.n = F.n / l;
                if (forced || (F.d >= -EPA_PLANE_EPS)) return face;
                status = 3;  // NonConvex
            } else {
                status = 2;  // Degenerated
            }
            remove(hull, face);
            append(stock, face);
            return -1;
        }
        status = stock.root >= 0 ? 6 : 5;
        return -1;
    }
    int findbest() {
        int minf = hull.root;
        float mind = fc[minf].d * fc[minf].d;
        for (int f = fc[minf].l[1]; f >= 0; f = fc[f].l[1]) {
            const float sqd = fc[f].d * fc[f].d;
            if (sqd < mind) { minf = f; mind = sqd; }
        }
        return minf;
    }
    // EPA::expand (btGjkEpa2.cpp:912-948), recursion replaced by an explicit stack
    bool expand(const Solver& g, int pass, int w, int f0, int e0, int& hcf, int& hff, int& hnf) {
        static const int i1m3[] = {1, 2, 0};
        static const int i2m3[] = {2, 0, 1};
        struct Frame { int f, e, stage; };
        Frame st[EPA_MAX_FACES + 1];
        int sp = 0;
        st[sp++] = {f0, e0, 0};
        bool ret = false;
        while (sp > 0) {
            Frame& fr = st[sp - 1];
            Face& F = fc[fr.f];
            if (fr.stage == 0) {
                if (F.pass == pass) { ret = false; sp--; continue; }
                const int e1 = i1m3[fr.e];
                if ((dot(F.n, g.sv[w].w) - F.d) < -EPA_PLANE_EPS) {
                    int nf = newface(g, F.c[e1], F.c[fr.e], w, false);
                    if (nf >= 0) {
                        bind(nf, 0, fr.f, fr.e);
                        if (hcf >= 0) bind(hcf, 1, nf, 2);
                        else hff = nf;
                        hcf = nf;
                        ++hnf;
                        ret = true;
                    } else {
                        ret = false;
                    }
                    sp--;
                    continue;
                }
                F.pass = (uint8_t)pass;
                fr.stage = 1;
                const int cf = F.f[e1], ce = F.e[e1];
                st[sp++] = {cf, ce, 0};
                continue;
            }
            if (fr.stage == 1) {
                if (!ret) { sp--; continue; }
                fr.stage = 2;
                const int e2 = i2m3[fr.e];
                const int cf = F.f[e2], ce = F.e[e2];
                st[sp++] = {cf, ce, 0};
                continue;
            }
            if (ret) {
                remove(hull, fr.f);
                append(stock, fr.f);
            }
            sp--;
        }
        return ret;
    }
    // EPA::Evaluate (btGjkEpa2.cpp:651-783)
    int evaluate(Solver& g, V3 guess) {
        Simplex& sx = *g.simplex;
        if ((sx.rank > 1) && g.enclose_origin()) {
            while (hull.root >= 0) {
                int f = hull.root;
                remove(hull, f);
                append(stock, f);
            }
            status = 0;
            nextsv = 0;
            if (Solver::det(g.sv[sx.c[0]].w - g.sv[sx.c[3]].w, g.sv[sx.c[1]].w - g.sv[sx.c[3]].w,
                            g.sv[sx.c[2]].w - g.sv[sx.c[3]].w) < 0) {
                std::swap(sx.c[0], sx.c[1]);
                std::swap(sx.p[0], sx.p[1]);
            }
            int tetra[4];
            tetra[0] = newface(g, sx.c[0], sx.c[1], sx.c[2], true);
            tetra[1] = newface(g, sx.c[1], sx.c[0], sx.c[3], true);
            tetra[2] = newface(g, sx.c[2], sx.c[1], sx.c[3], true);
            tetra[3] = newface(g, sx.c[0], sx.c[2], sx.c[3], true);
            if (hull.count == 4) {
                int best = findbest();
                Face outer = fc[best];
                int pass = 0;
                bind(tetra[0], 0, tetra[1], 0);
                bind(tetra[0], 1, tetra[2], 0);
                bind(tetra[0], 2, tetra[3], 0);
                bind(tetra[1], 1, tetra[3], 2);
                bind(tetra[1], 2, tetra[2], 1);
                bind(tetra[2], 2, tetra[3], 1);
                status = 0;
                for (int iterations = 0; iterations < EPA_MAX_ITER; ++iterations) {
                    if (nextsv < EPA_MAX_VERTICES) {
                        int hcf = -1, hff = -1, hnf = 0;
                        const int w = 4 + nextsv++;
                        bool valid = true;
                        fc[best].pass = (uint8_t)(++pass);
                        g.getsupport(fc[best].n, g.sv[w]);
                        const float wdist = dot(fc[best].n, g.sv[w].w) - fc[best].d;
                        if (wdist > EPA_ACCURACY) {
                            for (int j = 0; (j < 3) && valid; ++j)
                                valid &= expand(g, pass, w, fc[best].f[j], fc[best].e[j], hcf, hff, hnf);
                            if (valid && (hnf >= 3)) {
                                bind(hcf, 1, hff, 2);
                                remove(hull, best);
                                append(stock, best);
                                best = findbest();
                                outer = fc[best];
                            } else {
                                status = 4;  // InvalidHull
                                break;
                            }
                        } else {
                            status = 7;  // AccuraryReached
                            break;
                        }
                    } else {
                        status = 6;  // OutOfVertices
                        break;
                    }
                }
                const V3 projection = outer.n * outer.d;
                normal = outer.n;
                depth = outer.d;
                result.rank = 3;
                result.c[0] = outer.c[0];
                result.c[1] = outer.c[1];
                result.c[2] = outer.c[2];
                result.p[0] = len(cross(g.sv[outer.c[1]].w - projection, g.sv[outer.c[2]].w - projection));
                result.p[1] = len(cross(g.sv[outer.c[2]].w - projection, g.sv[outer.c[0]].w - projection));
                result.p[2] = len(cross(g.sv[outer.c[0]].w - projection, g.sv[outer.c[1]].w - projection));
                const float sum = result.p[0] + result.p[1] + result.p[2];
                result.p[0] /= sum;
                result.p[1] /= sum;
                result.p[2] /= sum;
                return status;
            }
        }
        status = 8;  // FallBack
        normal = -guess;
        const float nl = len(normal);
        if (nl > 0) normal = normal / nl;
        else normal = V3(1, 0, 0);
        depth = 0;
        result.rank = 1;
        result.c[0] = sx.c[0];
        result.p[0] = 1;
        return status;
    }
};

// Initialize (btGjkEpa2.cpp:953-969)
inline void setup(Minkowski& m, const Convex& a, const Xf& ta, const Convex& b, const Xf& tb, bool margins) {
    m.a = &a;
    m.b = &b;
    m.to_b = transpose_times(tb.b, ta.b);
    m.b_to_a = xf_inverse_times(ta, tb);
    m.margins = margins;
}

// btGjkEpaSolver2::Penetration (btGjkEpa2.cpp:1011-1052); false unless GJK finds the origin inside
inline bool penetration(const Convex& a, const Xf& ta, const Convex& b, const Xf& tb, V3 guess, V3& wa, V3& wb,
                        V3& nrm) {
    static thread_local Solver g;
    static thread_local Epa e;
    setup(g.shape, a, ta, b, tb, true);
    int gs = g.evaluate(-guess);
    if (gs != 1) return false;
    e.init();
    int es = e.evaluate(g, -guess);
    if (es == 9) return false;
    V3 w0(0, 0, 0);
    for (int i = 0; i < e.result.rank; ++i) w0 += g.shape.sup(g.sv[e.result.c[i]].d, 0) * e.result.p[i];
    wa = xf_apply(ta, w0);
    wb = xf_apply(ta, w0 - e.normal * e.depth);
    nrm = -e.normal;
    return true;
}
// btGjkEpaSolver2::Distance (btGjkEpa2.cpp:979-1010)
inline bool distance(const Convex& a, const Xf& ta, const Convex& b, const Xf& tb, V3 guess, V3& wa, V3& wb,
                     V3& nrm) {
    static thread_local Solver g;
    setup(g.shape, a, ta, b, tb, false);
    int gs = g.evaluate(guess);
    if (gs != 0) return false;
    V3 w0(0, 0, 0), w1(0, 0, 0);
    for (int i = 0; i < g.simplex->rank; ++i) {
        const float p = g.simplex->p[i];
        w0 += g.shape.sup(g.sv[g.simplex->c[i]].d, 0) * p;
        w1 += g.shape.sup(-g.sv[g.simplex->c[i]].d, 1) * p;
    }
    wa = xf_apply(ta, w0);
    wb = xf_apply(ta, w1);
    nrm = w0 - w1;
    float dist = len(nrm);
    nrm = nrm / (dist > GJK_MIN_DISTANCE ? dist : 1);
    return true;
}
// btGjkEpaPenetrationDepthSolver::calcPenDepth (btGjkEpaPenetrationDepthSolver.cpp:22-77)
inline bool calc_pen_depth(const Convex& a, const Xf& ta, const Convex& b, const Xf& tb, V3& v, V3& wa, V3& wb) {
    const V3 guesses[] = {safe_normalized(tb.o - ta.o), safe_normalized(ta.o - tb.o), V3(0, 0, 1), V3(0, 1, 0),
                          V3(1, 0, 0), V3(1, 1, 0), V3(1, 1, 1), V3(0, 1, 1), V3(1, 0, 1)};
    for (const V3& gv : guesses) {
        V3 pa, pb, n;
        if (penetration(a, ta, b, tb, gv, pa, pb, n)) { wa = pa; wb = pb; v = n; return true; }
        if (distance(a, ta, b, tb, gv, pa, pb, n)) { wa = pa; wb = pb; v = n; return false; }
    }
    wa = wb = v = V3(0, 0, 0);
    return false;
}
}  // namespace epa

// result of one GJK query; `epa_needed` is set where the reference would run EPA
struct GjkOut {
    bool valid = false;
    V3 normal, point_on_b;
    float dist = 0;
    bool epa_needed = false;
};

GjkOut gjk(const Convex& A, const Xf& ta_in, const Convex& B, const Xf& tb_in, float max_dist2) {
    GjkOut out;
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
            float rlen = 1.f / std::sqrt(l2);
            normalInB *= rlen;
            float s = std::sqrt(sqd);
            pA -= sep * (mA / s);
            pB += sep * (mB / s);
            distance = ((1.f / rlen) - margin);
            is_valid = true;
        }
    }
    bool catch_deg = degenerate && ((distance + margin) < 0.01f);
    if (!is_valid || catch_deg) {
        // penetration depth (btGjkPairDetector.cpp:850-922)
        out.epa_needed = true;
        V3 sep_axis(0, 0, 0), tA, tB;
        bool valid2 = epa::calc_pen_depth(A, ta, B, tb, sep_axis, tA, tB);
        if (valid2) {
            V3 tn = tB - tA;
            float l2 = len2(tn);
            if (l2 <= SIMD_EPS * SIMD_EPS) {
                tn = sep_axis;
                l2 = len2(sep_axis);
            }
            if (l2 > SIMD_EPS * SIMD_EPS) {
                tn = tn / std::sqrt(l2);
                float d2 = -len(tA - tB);
                if (!is_valid || (d2 < distance)) {
                    distance = d2;
                    pA = tA;
                    pB = tB;
                    normalInB = tn;
                    is_valid = true;
                }
            }
        } else if (len2(sep_axis) > 0.f) {
            float d2 = len(tA - tB) - margin;
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
    if (is_valid && ((distance < 0) || (distance * distance < max_dist2))) {
        // m_fixContactNormalDirection
        V3 amn, amx, bmn, bmx;
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

// SphereTriangleDetector::collide (B/.../CollisionDispatch/SphereTriangleDetector.cpp:139-244)
bool sphere_triangle(V3 center, float radius, const V3 v[3], float threshold, V3& point, V3& normal_out, float& depth) {
    float rwt = radius + threshold;
    V3 n = cross(v[1] - v[0], v[2] - v[0]);
    float l2 = len2(n);
    bool has = false;
    V3 cpnt;
    if (l2 >= SIMD_EPS * SIMD_EPS) {
        n = n / std::sqrt(l2);
        V3 p1c = center - v[0];
        float dfp = dot(p1c, n);
        if (dfp < 0.f) { dfp *= -1.f; n *= -1.f; }
        if (dfp < rwt) {
            // pointInTriangle (barycentric variant, SphereTriangleDetector.cpp:246-281)
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
                float minsq = rwt * rwt;
                // closestPointTriangle (SphereTriangleDetector.cpp:87-128)
                V3 a = v[0], b = v[1], c = v[2], p = center;
                V3 ab = b - a, ac = c - a, ap = p - a;
                V3 res;
                float d1 = dot(ab, ap), d2 = dot(ac, ap);
                if (d1 <= 0.f && d2 <= 0.f) res = a;
                else {
                    V3 bp = p - b;
                    float d3 = dot(ab, bp), d4 = dot(ac, bp);
                    if (d3 >= 0.f && d4 <= d3) res = b;
                    else {
                        V3 cp = p - c;
                        float d5 = dot(ab, cp), d6 = dot(ac, cp);
                        if (d6 >= 0.f && d5 <= d6) res = c;
                        else {
                            float vc = d1 * d4 - d3 * d2;
                            if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) res = a + (d1 / (d1 - d3)) * ab;
                            else {
                                float vb = d5 * d2 - d1 * d6;
                                if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) res = a + (d2 / (d2 - d6)) * ac;
                                else {
                                    float va = d3 * d6 - d5 * d4;
                                    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f)
                                        res = b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b);
                                    else {
                                        float denom = 1.f / (va + vb + vc);
                                        float vv2 = vb * denom, ww = vc * denom;
                                        res = a + vv2 * ab + ww * ac;
                                    }
                                }
                            }
                        }
                    }
                }
                float dsq = len2(res - center);
                if (dsq < minsq) { has = true; cpnt = res; }
            }
        }
    }
    if (has) {
        V3 c2 = center - cpnt;
        float dsq = len2(c2);
        if (dsq < rwt * rwt) {
            if (dsq > SIMD_EPS) {
                float d = std::sqrt(dsq);
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

// btTransformAabb(min, max, margin 0, t) (B/LinearMath/btAabbUtil2.h:166-181)
void transform_aabb_mm(V3 mn, V3 mx, const Xf& t, V3& omn, V3& omx) {
    V3 lhe = 0.5f * (mx - mn), lc = 0.5f * (mx + mn);
    M3 ab = absolute(t.b);
    V3 c = xf_apply(t, lc);
    V3 e(dot(ab.r[0], lhe), dot(ab.r[1], lhe), dot(ab.r[2], lhe));
    omn = c - e;
    omx = c + e;
}
// btBoxBoxDetector (B/.../CollisionDispatch/btBoxBoxDetector.cpp:30-767), the ODE
// separating-axis box test, restated.  Boxes are (center, basis, half extents
// with margin); each contact is reported the way the detector feeds
// btManifoldResult::addContactPoint: normal on B = -n, point on B, depth.
struct BoxHit { V3 point; float depth; };

// column j of a basis dotted with v, in the detector's summation order
inline float col_dot(const M3& m, int j, V3 v) { return m.r[0][j] * v.x + m.r[1][j] * v.y + m.r[2][j] * v.z; }
inline float cols_dot(const M3& a, int i, const M3& b, int j) {
    return a.r[0][i] * b.r[0][j] + a.r[1][i] * b.r[1][j] + a.r[2][i] * b.r[2][j];
}

// dLineClosestApproach (btBoxBoxDetector.cpp:82-108)
void line_closest(V3 pa, V3 ua, V3 pb, V3 ub, float& alpha, float& beta) {
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

// intersectRectQuad2 (btBoxBoxDetector.cpp:118-175): clips the quad q[8] against the
// rectangle |x| < h[0], |y| < h[1]; returns the polygon (at most 8 points) in ret.
int clip_quad(const float h[2], const float quad[8], float ret[16]) {
    float bufA[16], bufB[16];
    for (int i = 0; i < 8; i++) bufA[i] = quad[i];
    float* q = bufA;
    float* r = ret;
    float* other = bufB;
    int nq = 4, nr = 0;
    bool full = false;
    for (int dir = 0; dir <= 1 && !full; dir++) {
        for (int sign = -1; sign <= 1 && !full; sign += 2) {
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
                float* nq_ = (i > 1) ? pq + 2 : q;
                bool nin = sign * nq_[dir] < h[dir];
                if (in != nin) {
                    pr[1 - dir] = pq[1 - dir] + (nq_[1 - dir] - pq[1 - dir]) / (nq_[dir] - pq[dir]) * (sign * h[dir] - pq[dir]);
                    pr[dir] = sign * h[dir];
                    pr += 2;
                    nr++;
                    if (nr & 8) { full = true; break; }
                }
                pq += 2;
            }
            if (full) { q = r; break; }
            // the chopped polygon becomes the input of the next pass
            q = r;
            if (r == ret) { r = other; }
            else { r = ret; }
            nq = nr;
        }
    }
    if (q != ret)
        for (int i = 0; i < nr * 2; i++) ret[i] = q[i];
    return nr;
}

// cullPoints2 (btBoxBoxDetector.cpp:187-245): picks m of n polygon points spread by angle
void cull_points(int n, const float p[], int m, int i0, int iret[]) {
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
        if (std::fabs(a + q) > SIMD_EPS) a = 1.f / (3.0f * (a + q));
        else a = BT_LARGE;
        cx = a * (cx + q * (p[n * 2 - 2] + p[0]));
        cy = a * (cy + q * (p[n * 2 - 1] + p[1]));
    }
    float ang[8];
    for (int i = 0; i < n; i++) ang[i] = std::atan2(p[i * 2 + 1] - cy, p[i * 2] - cx);
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
                float diff = std::fabs(ang[i] - a);
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

// dBoxBox2 (btBoxBoxDetector.cpp:247-712) with maxc = 4.  Returns the contact count;
// `normal` is the detector's normal (contacts go in with -normal).
int box_box(V3 p1, const M3& R1, V3 A, V3 p2, const M3& R2, V3 B, V3& normal, BoxHit out[4]) {
    const float fudge_factor = 1.05f;
    V3 p(p2.x - p1.x, p2.y - p1.y, p2.z - p1.z);
    float pp[3] = {col_dot(R1, 0, p), col_dot(R1, 1, p), col_dot(R1, 2, p)};
    float Rm[3][3], Q[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            Rm[i][j] = cols_dot(R1, i, R2, j);
            Q[i][j] = std::fabs(Rm[i][j]);
        }
    float s = -FLT_MAX, s2, l;
    int normal_axis = -1;  // >= 0: column of R1 (0..2) or R2 (3..5)
    V3 normalC(0.f, 0.f, 0.f);
    bool invert = false;
    int code = 0;
    auto face = [&](float e1, float e2, int axis, int cc) -> bool {
        s2 = std::fabs(e1) - e2;
        if (s2 > 0) return false;
        if (s2 > s) {
            s = s2;
            normal_axis = axis;
            invert = e1 < 0;
            code = cc;
        }
        return true;
    };
    const float* Av = &A.x;
    const float* Bv = &B.x;
    if (!face(pp[0], A.x + B.x * Q[0][0] + B.y * Q[0][1] + B.z * Q[0][2], 0, 1)) return 0;
    if (!face(pp[1], A.y + B.x * Q[1][0] + B.y * Q[1][1] + B.z * Q[1][2], 1, 2)) return 0;
    if (!face(pp[2], A.z + B.x * Q[2][0] + B.y * Q[2][1] + B.z * Q[2][2], 2, 3)) return 0;
    if (!face(col_dot(R2, 0, p), A.x * Q[0][0] + A.y * Q[1][0] + A.z * Q[2][0] + B.x, 3, 4)) return 0;
    if (!face(col_dot(R2, 1, p), A.x * Q[0][1] + A.y * Q[1][1] + A.z * Q[2][1] + B.y, 4, 5)) return 0;
    if (!face(col_dot(R2, 2, p), A.x * Q[0][2] + A.y * Q[1][2] + A.z * Q[2][2] + B.z, 5, 6)) return 0;
    auto edge = [&](float e1, float e2, float n1, float n2, float n3, int cc) -> bool {
        s2 = std::fabs(e1) - e2;
        if (s2 > SIMD_EPS) return false;
        l = std::sqrt(n1 * n1 + n2 * n2 + n3 * n3);
        if (l > SIMD_EPS) {
            s2 /= l;
            if (s2 * fudge_factor > s) {
                s = s2;
                normal_axis = -1;
                normalC = V3(n1 / l, n2 / l, n3 / l);
                invert = e1 < 0;
                code = cc;
            }
        }
        return true;
    };
    const float f2 = 1.0e-5f;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Q[i][j] += f2;
    const float (&R)[3][3] = Rm;
    // u1 x (v1, v2, v3)
    if (!edge(pp[2] * R[1][0] - pp[1] * R[2][0], A.y * Q[2][0] + A.z * Q[1][0] + B.y * Q[0][2] + B.z * Q[0][1], 0, -R[2][0], R[1][0], 7)) return 0;
    if (!edge(pp[2] * R[1][1] - pp[1] * R[2][1], A.y * Q[2][1] + A.z * Q[1][1] + B.x * Q[0][2] + B.z * Q[0][0], 0, -R[2][1], R[1][1], 8)) return 0;
    if (!edge(pp[2] * R[1][2] - pp[1] * R[2][2], A.y * Q[2][2] + A.z * Q[1][2] + B.x * Q[0][1] + B.y * Q[0][0], 0, -R[2][2], R[1][2], 9)) return 0;
    // u2 x (v1, v2, v3)
    if (!edge(pp[0] * R[2][0] - pp[2] * R[0][0], A.x * Q[2][0] + A.z * Q[0][0] + B.y * Q[1][2] + B.z * Q[1][1], R[2][0], 0, -R[0][0], 10)) return 0;
    if (!edge(pp[0] * R[2][1] - pp[2] * R[0][1], A.x * Q[2][1] + A.z * Q[0][1] + B.x * Q[1][2] + B.z * Q[1][0], R[2][1], 0, -R[0][1], 11)) return 0;
    if (!edge(pp[0] * R[2][2] - pp[2] * R[0][2], A.x * Q[2][2] + A.z * Q[0][2] + B.x * Q[1][1] + B.y * Q[1][0], R[2][2], 0, -R[0][2], 12)) return 0;
    // u3 x (v1, v2, v3)
    if (!edge(pp[1] * R[0][0] - pp[0] * R[1][0], A.x * Q[1][0] + A.y * Q[0][0] + B.y * Q[2][2] + B.z * Q[2][1], -R[1][0], R[0][0], 0, 13)) return 0;
    if (!edge(pp[1] * R[0][1] - pp[0] * R[1][1], A.x * Q[1][1] + A.y * Q[0][1] + B.x * Q[2][2] + B.z * Q[2][0], -R[1][1], R[0][1], 0, 14)) return 0;
    if (!edge(pp[1] * R[0][2] - pp[0] * R[1][2], A.x * Q[1][2] + A.y * Q[0][2] + B.x * Q[2][1] + B.y * Q[2][0], -R[1][2], R[0][2], 0, 15)) return 0;
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
    if (code > 6) {
        // edge-edge: closest points of the two touching edges
        V3 pa = p1;
        for (int j = 0; j < 3; j++) {
            float sign = (col_dot(R1, j, normal) > 0) ? 1.0f : -1.0f;
            for (int i = 0; i < 3; i++) pa[i] += sign * Av[j] * R1.r[i][j];
        }
        V3 pb = p2;
        for (int j = 0; j < 3; j++) {
            float sign = (col_dot(R2, j, normal) > 0) ? -1.0f : 1.0f;
            for (int i = 0; i < 3; i++) pb[i] += sign * Bv[j] * R2.r[i][j];
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
    // face contact: reference face a, incident face b
    const M3& Ra = code <= 3 ? R1 : R2;
    const M3& Rb = code <= 3 ? R2 : R1;
    V3 pa = code <= 3 ? p1 : p2, pb = code <= 3 ? p2 : p1;
    const float* Sa = code <= 3 ? Av : Bv;
    const float* Sb = code <= 3 ? Bv : Av;
    V3 normal2 = code <= 3 ? normal : V3(-normal.x, -normal.y, -normal.z);
    float nr[3] = {col_dot(Rb, 0, normal2), col_dot(Rb, 1, normal2), col_dot(Rb, 2, normal2)};
    float anr[3] = {std::fabs(nr[0]), std::fabs(nr[1]), std::fabs(nr[2])};
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
    int codeN = code <= 3 ? code - 1 : code - 4;
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
    int maxc = 4;
    if (maxc > cnum) maxc = cnum;
    auto emit = [&](int k, int j) {
        V3 w(point[j * 3] + pa.x, point[j * 3 + 1] + pa.y, point[j * 3 + 2] + pa.z);
        if (code >= 4) w = w - normal * dep[j];
        out[k].point = w;
        out[k].depth = dep[j];
    };
    if (cnum <= maxc) {
        for (int j = 0; j < cnum; j++) emit(j, j);
        return cnum;
    }
    int i1 = 0;
    float maxdepth = dep[0];
    for (int i = 1; i < cnum; i++)
        if (dep[i] > maxdepth) { maxdepth = dep[i]; i1 = i; }
    int iret[8];
    cull_points(cnum, ret, maxc, i1, iret);
    for (int j = 0; j < maxc; j++) emit(j, iret[j]);
    return maxc;
}

// ================================================================ collision dispatch
struct PairRec { int o0, o1; };  // o0 has the lower broadphase uid

struct World {
    std::vector<Manifold> manifolds;
};

// Contact-added callback (Arena::_BulletContactAddedCallback, Arena.cpp:244-414) for
// a point stored in manifold m at index idx; `tri` is the mesh triangle or -1.
void contact_added(Arena& a, Manifold& m, int idx, int tri) {
    MPoint& cp = m.pts[idx];
    int A = m.body0, B = m.body1;
    auto user_index = [&](int o) { return o == OBJ_BALL ? 2 : (o >= OBJ_CAR0 ? 1 : -1); };
    auto responds = [&](int o) { return a.is_static(o) ? true : !a.body(o).no_contact_response; };
    if (!responds(A) || !responds(B)) return;
    int ua = user_index(A), ub = user_index(B);
    bool swap;
    if (ua != -1 && ub != -1) swap = ua > ub;
    else swap = ub != -1;
    if (swap) { std::swap(A, B); std::swap(ua, ub); }
    if (ua == 1) {
        Car& car = a.cars[A - OBJ_CAR0];
        if (ub == 2) {
            // car-ball: Ball::_OnHit (Ball.cpp:237-289)
            V3 rel_ball = (swap ? cp.local_a : cp.local_b) * BT_TO_UU;
            car_refresh_state(car);
            rsg_ball_state bst;
            get_ball_state(a, bst);
            cp.friction = RL::CARBALL_COLLISION_FRICTION;
            cp.restitution = RL::CARBALL_COLLISION_RESTITUTION;
            rsg_ball_hit_info& bhi = car.st.ball_hit_info;
            bhi.is_valid = 1;
            bhi.relative_pos_on_ball = P(rel_ball);
            bhi.tick_count_when_hit = a.tick_count;
            bhi.ball_pos = bst.pos;
            bhi.extra_hit_vel = {0, 0, 0};
            a.events.push_back({RSG_EVENT_BALL_HIT, a.tick_count, car.id, 0, 0});
            if ((a.tick_count > bhi.tick_count_when_extra_impulse_applied + 1) ||
                (bhi.tick_count_when_extra_impulse_applied > a.tick_count)) {
                bhi.tick_count_when_extra_impulse_applied = a.tick_count;
                V3 cf = V(car.st.rot_mat.forward);
                V3 rel_pos = V(bst.pos) - V(car.st.pos);
                V3 rel_vel = V(bst.vel) - V(car.st.vel);
                float rs = rs_min(rs_len(rel_vel), RL::BALL_CAR_EXTRA_IMPULSE_MAXDELTAVEL_UU);
                if (rs > 0) {
                    V3 hit = rs_normalized(rel_pos * V3(1, 1, RL::BALL_CAR_EXTRA_IMPULSE_Z_SCALE));
                    V3 adj = cf * dot(hit, cf) * (1 - RL::BALL_CAR_EXTRA_IMPULSE_FORWARD_SCALE);
                    hit = rs_normalized(hit - adj);
                    V3 added = (hit * rs) * BALL_CAR_EXTRA_IMPULSE_FACTOR.eval(rs) * 1.f;
                    bhi.extra_hit_vel = P(added);
                    a.ball_cache += added * UU_TO_BT;
                }
            }
        } else if (ub == 1) {
            // car-car: Arena::_BtCallback_OnCarCarCollision (Arena.cpp:323-405)
            Car* c1 = &car;
            Car* c2 = &a.cars[B - OBJ_CAR0];
            cp.friction = RL::CARCAR_COLLISION_FRICTION;
            cp.restitution = RL::CARCAR_COLLISION_RESTITUTION;
            for (int i = 0; i < 2; i++) {
                bool sw = i == 1;
                if (sw) std::swap(c1, c2);
                car_refresh_state(*c1);
                car_refresh_state(*c2);
                rsg_car_state& s = c1->st;
                rsg_car_state& o = c2->st;
                if (s.is_demoed || o.is_demoed) return;
                if (s.car_contact_other_car_id == c2->id && s.car_contact_cooldown_timer > 0) continue;
                V3 dp = V(o.pos) - V(s.pos);
                if (dot(V(s.vel), dp) > 0) {
                    V3 vd = rs_normalized(V(s.vel));
                    V3 dir = rs_normalized(dp);
                    float sto = dot(V(s.vel), dir);
                    float oas = dot(V(o.vel), vd);
                    if (sto > oas) {
                        V3 lp = sw ? cp.local_b : cp.local_a;
                        bool bumper = (lp.x * BT_TO_UU) > RL::BUMP_MIN_FORWARD_DIST;
                        if (bumper) {
                            bool demo = s.is_supersonic;
                            if (demo) demo = c1->team != c2->team;
                            if (demo) {
                                o.is_demoed = 1;
                                o.demo_respawn_timer = RL::DEMO_RESPAWN_TIME;
                            } else {
                                bool gh = o.is_on_ground;
                                float bs = (gh ? BUMP_VEL_AMOUNT_GROUND : BUMP_VEL_AMOUNT_AIR).eval(sto);
                                V3 hu = o.is_on_ground ? V(o.rot_mat.up) : V3(0, 0, 1);
                                V3 bi = vd * bs + hu * BUMP_UPWARD_VEL_AMOUNT.eval(sto) * 1.f;
                                c2->vel_impulse_cache += bi * UU_TO_BT;
                            }
                            s.car_contact_other_car_id = c2->id;
                            s.car_contact_cooldown_timer = RL::BUMP_COOLDOWN_TIME;
                            a.events.push_back({RSG_EVENT_BUMP, a.tick_count, c1->id, c2->id, (uint32_t)demo});
                        }
                    }
                }
            }
        } else {
            // car-world (Arena.cpp:407-414)
            car.st.world_contact_has_contact = 1;
            car.st.world_contact_normal = P(cp.normal);
            cp.friction = RL::CARWORLD_COLLISION_FRICTION;
            cp.restitution = RL::CARWORLD_COLLISION_RESTITUTION;
        }
    } else if (ua == 2 && ub == -1) {
        cp.special = true;  // ball-world (Arena.cpp:298-306)
    }
    if (tri >= 0) adjust_internal_edge(cp, tri);
}

float combined_friction(Arena& a, int o0, int o1) {  // btManifoldResult::calculateCombinedFriction (RocketSim variant)
    auto fr = [&](int o) { return a.is_static(o) ? RL::ARENA_COLLISION_BASE_FRICTION : a.body(o).friction; };
    float x = fr(o0), y = fr(o1);
    if (a.is_static(o0) || a.is_static(o1)) return x < y ? x : y;
    return x * y;
}
float combined_restitution(Arena& a, int o0, int o1) {
    auto re = [&](int o) { return a.is_static(o) ? RL::ARENA_COLLISION_BASE_RESTITUTION : a.body(o).restitution; };
    float x = re(o0), y = re(o1);
    if (a.is_static(o0) || a.is_static(o1)) return x > y ? x : y;
    return x * y;
}

Xf obj_xf(Arena& a, int o) {
    if (o == OBJ_MESH) return xf_identity();
    if (o < OBJ_BALL) { Xf t = xf_identity(); t.o = a.planes[o - OBJ_PLANE0].origin; return t; }
    return a.body(o).xf;
}

// convex object (ball sphere or car box) against the mesh: btConvexConcaveCollisionAlgorithm
// (btConvexConcaveCollisionAlgorithm.cpp:71-250) with per-triangle sphere-triangle or GJK
void convex_vs_mesh(Arena& a, Manifold& m, int conv, const Xf& conv_xf, const Convex& cshape) {
    const Mesh& mesh = *g_mesh;
    V3 mn, mx;
    cshape.aabb(conv_xf, mn, mx);  // convex AABB in mesh space (identity)
    // m_aabbMin/Max extended by triangle margin (0) + closest-point threshold (0)
    Xf mesh_xf = xf_identity();
    Xf x0 = a.body(m.body0).xf, x1 = obj_xf(a, m.body1);
    float fr = combined_friction(a, OBJ_MESH, conv), re = combined_restitution(a, OBJ_MESH, conv);
    mesh.query_aabb(mn, mx, [&](int t) {
        V3 tv[3];
        mesh.tri_verts(t, tv);
        // TestTriangleAgainstAabb2 (z, x, y)
        const int ord[3] = {2, 0, 1};
        for (int k : ord) {
            if (std::min(std::min(tv[0][k], tv[1][k]), tv[2][k]) > mx[k]) return;
            if (std::max(std::max(tv[0][k], tv[1][k]), tv[2][k]) < mn[k]) return;
        }
        // early out on the triangle normal (BT_DISABLE_CONVEX_CONCAVE_EARLY_OUT not set)
        {
            V3 tn = normalized(cross(tv[1] - tv[0], tv[2] - tv[0]));
            float thr = m.breaking;
            for (int side = 0; side < 2; side++) {
                V3 dir = side ? -tn : tn;
                V3 ld = inverse(conv_xf.b) * dir;  // basis.inverse() * n
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
                if (pt - pp > thr) return;
            }
        }
        if (cshape.type == 1) {
            // btSphereTriangleCollisionAlgorithm (swapResults=false), sphere is A
            V3 point, nrm;
            float depth;
            V3 center = xf_inv_apply(mesh_xf, conv_xf.o);
            if (sphere_triangle(center, cshape.margin, tv, m.breaking, point, nrm, depth)) {
                a.counters[1]++;
                int idx = add_point(a, m, x0, x1, nrm, point, depth, true, fr, re);
                if (idx >= 0) contact_added(a, m, idx, t);
            }
        } else {
            Convex tri;
            tri.type = 2;
            tri.margin = 0.f;
            for (int k = 0; k < 3; k++) tri.tv[k] = tv[k];
            float md = cshape.margin + tri.margin + m.breaking;
            GjkOut g = gjk(cshape, conv_xf, tri, mesh_xf, md * md);
            a.counters[2]++;
            if (g.epa_needed) a.counters[3]++;
            if (g.valid) {
                int idx = add_point(a, m, x0, x1, g.normal, g.point_on_b, g.dist, true, fr, re);
                if (idx >= 0) contact_added(a, m, idx, t);
            }
        }
    });
    refresh(m, x0, x1);
}

// convex vs plane: btConvexPlaneCollisionAlgorithm::processCollision (btConvexPlaneCollisionAlgorithm.cpp:94-161)
void convex_vs_plane(Arena& a, Manifold& m, const Xf& conv_xf, const Convex& cshape, int plane_obj) {
    const Plane& pl = a.planes[plane_obj - OBJ_PLANE0];
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
    float distance = dot(pl.n, vip) - pl.c;
    bool has = distance < m.breaking;
    Xf x0 = a.body(m.body0).xf, x1 = pxf;
    if (has) {
        V3 proj = vip - distance * pl.n;
        V3 pw = xf_apply(pxf, proj);
        V3 nw = pxf.b * pl.n;
        int conv = m.body0;
        float fr = combined_friction(a, plane_obj, conv), re = combined_restitution(a, plane_obj, conv);
        int idx = add_point(a, m, x0, x1, nw, pw, distance, true, fr, re);
        a.counters[4]++;
        if (idx >= 0) contact_added(a, m, idx, -1);
    }
    if (m.n) refresh(m, x0, x1);
}

// Bullet's btAlignedObjectArray::quickSortInternal (B/LinearMath/btAlignedObjectArray.h)
template <class T, class L>
void bt_quicksort(std::vector<T>& v, L less, int lo, int hi) {
    int i = lo, j = hi;
    T x = v[(lo + hi) / 2];
    do {
        while (less(v[i], x)) i++;
        while (less(x, v[j])) j--;
        if (i <= j) { std::swap(v[i], v[j]); i++; j--; }
    } while (i <= j);
    if (lo < j) bt_quicksort(v, less, lo, j);
    if (i < hi) bt_quicksort(v, less, i, hi);
}

// ================================================================ solver
// btSequentialImpulseConstraintSolver (B/BulletDynamics/ConstraintSolver/btSequentialImpulseConstraintSolver.cpp)
struct SBody {
    int obj = -1;  // -1 fixed body
    V3 dlv, dav, push, turn;
    V3 inv_mass;
    V3 lv, av, ext_f, ext_t;
    Xf xf;
};
struct Row {
    int ba, bb;
    V3 n1, n2, rp1xn, rp2xn, angA, angB;
    float jac_inv = 0, rhs = 0, rhs_pen = 0, cfm = 0, lo = 0, hi = 0, applied = 0, applied_push = 0, friction = 0;
    int friction_index = 0;
    bool special = false;
};

struct Solver {
    std::vector<SBody> bodies;
    std::vector<Row> contacts, frictions;
    int fixed_id = -1;
};

int get_solver_body(Arena& a, Solver& s, int obj, float dt) {
    if (obj >= 0 && !a.is_static(obj)) {
        for (size_t i = 0; i < s.bodies.size(); i++)
            if (s.bodies[i].obj == obj) return (int)i;
        Body& b = a.body(obj);
        SBody sb;
        sb.obj = obj;
        sb.xf = b.xf;
        sb.inv_mass = V3(b.inv_mass, b.inv_mass, b.inv_mass);
        sb.lv = b.lin_vel;
        sb.av = b.ang_vel;
        sb.ext_f = b.total_force * b.inv_mass * dt;
        sb.ext_t = b.total_torque * b.inv_inertia_world * dt;
        s.bodies.push_back(sb);
        return (int)s.bodies.size() - 1;
    }
    if (s.fixed_id < 0) {
        SBody sb;
        sb.obj = -1;
        sb.xf = xf_identity();
        s.bodies.push_back(sb);
        s.fixed_id = (int)s.bodies.size() - 1;
    }
    return s.fixed_id;
}

void setup_contact_row(Arena& a, Solver& s, Row& r, int ia, int ib, const MPoint& cp, V3 rel1, V3 rel2, float dt) {
    SBody& A = s.bodies[ia];
    SBody& B = s.bodies[ib];
    Body* rb0 = A.obj >= 0 ? &a.body(A.obj) : nullptr;
    Body* rb1 = B.obj >= 0 ? &a.body(B.obj) : nullptr;
    float relax = 1.f;
    float inv_dt = 1.f / dt;
    float cfm = 0.f * inv_dt;
    float erp = 0.8f;  // m_erp2 (Arena.cpp:473-475)
    V3 ta0 = cross(rel1, cp.normal);
    r.angA = rb0 ? rb0->inv_inertia_world * ta0 : V3(0, 0, 0);
    V3 ta1 = cross(rel2, cp.normal);
    r.angB = rb1 ? rb1->inv_inertia_world * (-ta1) : V3(0, 0, 0);
    float d0 = 0, d1 = 0;
    if (rb0) { V3 v = cross(r.angA, rel1); d0 = rb0->inv_mass + dot(cp.normal, v); }
    if (rb1) { V3 v = cross(-r.angB, rel2); d1 = rb1->inv_mass + dot(cp.normal, v); }
    r.jac_inv = relax / (d0 + d1 + cfm);
    if (rb0) { r.n1 = cp.normal; r.rp1xn = ta0; } else { r.n1 = V3(0, 0, 0); r.rp1xn = V3(0, 0, 0); }
    if (rb1) { r.n2 = -cp.normal; r.rp2xn = -ta1; } else { r.n2 = V3(0, 0, 0); r.rp2xn = V3(0, 0, 0); }
    float restitution = 0.f;
    float penetration = cp.dist + 0.f;
    {
        V3 v1 = rb0 ? rb0->vel_at(rel1) : V3(0, 0, 0);
        V3 v2 = rb1 ? rb1->vel_at(rel2) : V3(0, 0, 0);
        float rel_vel = dot(cp.normal, v1 - v2);
        r.friction = cp.friction;
        // restitutionCurve (threshold 0.2)
        if (std::fabs(rel_vel) < 0.2f) restitution = 0.f;
        else restitution = cp.restitution * -rel_vel;
        if (restitution <= 0.f) restitution = 0.f;
    }
    // warm starting: manifolds are new every tick so the cached impulse is 0
    r.applied = 0.f * 0.85f;
    r.applied_push = 0.f;
    {
        V3 efA = A.obj >= 0 ? A.ext_f : V3(0, 0, 0), etA = A.obj >= 0 ? A.ext_t : V3(0, 0, 0);
        V3 efB = B.obj >= 0 ? B.ext_f : V3(0, 0, 0), etB = B.obj >= 0 ? B.ext_t : V3(0, 0, 0);
        float v1 = dot(r.n1, A.lv + efA) + dot(r.rp1xn, A.av + etA);
        float v2 = dot(r.n2, B.lv + efB) + dot(r.rp2xn, B.av + etB);
        float rel_vel = v1 + v2;
        float pos_err = 0.f;
        float vel_err = restitution - rel_vel;
        if (penetration > 0) pos_err = 0;
        else pos_err = -penetration * erp * inv_dt;
        float pen_imp = pos_err * r.jac_inv;
        float vel_imp = vel_err * r.jac_inv;
        // split impulse: threshold 1e30 (Arena.cpp:474)
        if (!(true) || (penetration > 1.0e30f)) {
            r.rhs = pen_imp + vel_imp;
            r.rhs_pen = 0.f;
        } else {
            r.rhs = vel_imp;
            r.rhs_pen = pen_imp;
        }
        r.cfm = cfm * r.jac_inv;
        r.lo = 0;
        r.hi = 1e10f;
    }
    r.special = cp.special;
}

void setup_friction_row(Arena& a, Solver& s, Row& r, V3 n, int ia, int ib, const MPoint& cp, V3 rel1, V3 rel2) {
    SBody& A = s.bodies[ia];
    SBody& B = s.bodies[ib];
    Body* b0 = A.obj >= 0 ? &a.body(A.obj) : nullptr;
    Body* b1 = B.obj >= 0 ? &a.body(B.obj) : nullptr;
    r.ba = ia;
    r.bb = ib;
    r.friction = cp.friction;
    r.applied = 0;
    r.applied_push = 0;
    if (b0) {
        r.n1 = n;
        V3 t = cross(rel1, r.n1);
        r.rp1xn = t;
        r.angA = b0->inv_inertia_world * t;
    } else {
        r.n1 = r.rp1xn = r.angA = V3(0, 0, 0);
    }
    if (b1) {
        r.n2 = -n;
        V3 t = cross(rel2, r.n2);
        r.rp2xn = t;
        r.angB = b1->inv_inertia_world * t;
    } else {
        r.n2 = r.rp2xn = r.angB = V3(0, 0, 0);
    }
    float d0 = 0, d1 = 0;
    if (b0) { V3 v = cross(r.angA, rel1); d0 = b0->inv_mass + dot(n, v); }
    if (b1) { V3 v = cross(-r.angB, rel2); d1 = b1->inv_mass + dot(n, v); }
    r.jac_inv = 1.f / (d0 + d1);
    float v1 = dot(r.n1, b0 ? A.lv + A.ext_f : V3(0, 0, 0)) + dot(r.rp1xn, b0 ? A.av : V3(0, 0, 0));
    float v2 = dot(r.n2, b1 ? B.lv + B.ext_f : V3(0, 0, 0)) + dot(r.rp2xn, b1 ? B.av : V3(0, 0, 0));
    float rel_vel = v1 + v2;
    float vel_err = 0.f - rel_vel;
    float vel_imp = vel_err * r.jac_inv;
    r.rhs = 0.f + vel_imp;
    r.rhs_pen = 0.f;
    r.cfm = 0.f;
    r.lo = -r.friction;
    r.hi = r.friction;
}

// convertContactInner friction part (btSequentialImpulseConstraintSolver.cpp:1071-1162)
void add_friction(Arena& a, Solver& s, int ia, int ib, const MPoint& cp, V3 rel1, V3 rel2, int fidx) {
    SBody& A = s.bodies[ia];
    SBody& B = s.bodies[ib];
    V3 v1 = A.obj >= 0 ? A.lv + A.ext_f + cross(A.av + A.ext_t, rel1) : V3(0, 0, 0);
    V3 v2 = B.obj >= 0 ? B.lv + B.ext_f + cross(B.av + B.ext_t, rel2) : V3(0, 0, 0);
    V3 vel = v1 - v2;
    float rel_vel = dot(cp.normal, vel);
    V3 lat = vel - cp.normal * rel_vel;
    float lat2 = len2(lat);
    V3 dir;
    if (lat2 > SIMD_EPS) {
        dir = lat * (1.f / std::sqrt(lat2));
    } else {
        V3 d2;
        plane_space(cp.normal, dir, d2);
    }
    Row fr;
    fr.friction_index = fidx;
    setup_friction_row(a, s, fr, dir, ia, ib, cp, rel1, rel2);
    s.frictions.push_back(fr);
}

void solve_row(Solver& s, Row& c, bool lower_only) {  // gResolveSingleConstraintRow{Generic,LowerLimit}
    SBody& A = s.bodies[c.ba];
    SBody& B = s.bodies[c.bb];
    float d = c.rhs - c.applied * c.cfm;
    float d1 = simd_dot(c.n1, A.dlv) + simd_dot(c.rp1xn, A.dav);
    float d2 = simd_dot(c.n2, B.dlv) + simd_dot(c.rp2xn, B.dav);
    d -= d1 * c.jac_inv;
    d -= d2 * c.jac_inv;
    float sum = c.applied + d;
    if (sum < c.lo) { d = c.lo - c.applied; c.applied = c.lo; }
    else if (!lower_only && sum > c.hi) { d = c.hi - c.applied; c.applied = c.hi; }
    else c.applied = sum;
    if (A.obj >= 0) { A.dlv += c.n1 * A.inv_mass * d; A.dav += c.angA * d; }
    if (B.obj >= 0) { B.dlv += c.n2 * B.inv_mass * d; B.dav += c.angB * d; }
}

float solve_split(Solver& s, Row& c) {  // gResolveSplitPenetrationImpulse_sse2
    if (!c.rhs_pen) return 0.f;
    SBody& A = s.bodies[c.ba];
    SBody& B = s.bodies[c.bb];
    float d = c.rhs_pen - c.applied_push * c.cfm;
    float d1 = simd_dot(c.n1, A.push) + simd_dot(c.rp1xn, A.turn);
    float d2 = simd_dot(c.n2, B.push) + simd_dot(c.rp2xn, B.turn);
    d -= d1 * c.jac_inv;
    d -= d2 * c.jac_inv;
    float sum = c.applied_push + d;
    if (sum < c.lo) { d = c.lo - c.applied_push; c.applied_push = c.lo; }
    else c.applied_push = sum;
    if (A.obj >= 0) { A.push += c.n1 * A.inv_mass * d; A.turn += c.angA * d; }
    if (B.obj >= 0) { B.push += c.n2 * B.inv_mass * d; B.turn += c.angB * d; }
    return (float)(d * (1. / c.jac_inv));
}

void convert_contact_point(Arena& a, Solver& s, int o0, int o1, const MPoint& cp, int ia, int ib, float dt) {
    Row r;
    r.ba = ia;
    r.bb = ib;
    V3 rel1 = cp.pos_a - obj_xf(a, o0).o;
    V3 rel2 = cp.pos_b - obj_xf(a, o1).o;
    setup_contact_row(a, s, r, ia, ib, cp, rel1, rel2, dt);
    r.friction_index = (int)s.frictions.size();
    if (cp.special) {
        for (int i = 0; i < 2; i++) {
            int o = i ? o1 : o0;
            if (!a.is_static(o)) {
                Body& b = a.body(o);
                b.n_special++;
                b.sp_friction = cp.friction;
                b.sp_restitution = cp.restitution;
                b.sp_total_normal += cp.normal;
                b.sp_total_dist += len(i ? rel2 : rel1);
            }
        }
    }
    int fidx = (int)s.contacts.size();
    s.contacts.push_back(r);
    add_friction(a, s, ia, ib, cp, rel1, rel2, fidx);
}

void solve(Arena& a, std::vector<int>& bodies, std::vector<Manifold*>& mans, float dt) {
    Solver s;
    for (int o : bodies) {
        Body& b = a.body(o);
        if (b.inv_mass != 0.f) get_solver_body(a, s, o, dt);
        else get_solver_body(a, s, o, dt);
    }
    for (Manifold* m : mans) {
        int ia = get_solver_body(a, s, m->body0, dt);
        int ib = get_solver_body(a, s, m->body1, dt);
        bool a_fixed = s.bodies[ia].obj < 0, b_fixed = s.bodies[ib].obj < 0;
        if (a_fixed && b_fixed) continue;
        for (int j = 0; j < m->n; j++) {
            const MPoint& cp = m->pts[j];
            if (cp.dist <= BT_LARGE) convert_contact_point(a, s, m->body0, m->body1, cp, ia, ib, dt);
        }
    }
    // special contacts (convertContactSpecial, btSequentialImpulseConstraintSolver.cpp:1164-1211)
    for (int o : bodies) {
        Body& b = a.body(o);
        if (b.n_special > 0) {
            float dist = b.sp_total_dist / b.n_special;
            V3 nrm = b.sp_total_normal / (float)b.n_special;
            MPoint tmp;
            tmp.dist = dist;
            tmp.normal = nrm;
            tmp.friction = b.sp_friction;
            tmp.restitution = b.sp_restitution;
            int ia = get_solver_body(a, s, o, dt);
            if (s.fixed_id < 0) get_solver_body(a, s, -1, dt);
            int ib = s.fixed_id;
            Row r;
            r.ba = ia;
            r.bb = ib;
            V3 rel1 = nrm * -dist, rel2(0, 0, 0);
            setup_contact_row(a, s, r, ia, ib, tmp, rel1, rel2, dt);
            int fidx = (int)s.contacts.size();
            r.friction_index = (int)s.frictions.size();
            s.contacts.push_back(r);
            add_friction(a, s, ia, ib, tmp, rel1, rel2, fidx);
            b.n_special = 0;
            b.sp_friction = b.sp_restitution = b.sp_total_dist = 0;
            b.sp_total_normal = V3(0, 0, 0);
        }
    }
    a.counters[7] += s.contacts.size();  // workload statistics: solver rows per tick
    a.counters[8] += s.frictions.size();
    a.counters[9] += mans.size();
    const int ITER = 10;
    for (int it = 0; it < ITER; it++) {
        float lsr = 0;
        for (Row& c : s.contacts) {
            float res = solve_split(s, c);
            lsr = std::max(lsr, res * res);
        }
        if (lsr <= 0.f || it >= ITER - 1) break;
    }
    for (int it = 0; it < ITER; it++) {
        for (Row& c : s.contacts) {
            if (c.special) continue;
            solve_row(s, c, true);
        }
        for (Row& f : s.frictions) {
            float total = s.contacts[f.friction_index].applied;
            if (total > 0.f) {
                f.lo = -(f.friction * total);
                f.hi = f.friction * total;
                solve_row(s, f, false);
            }
        }
    }
    // writeBackBodies (btSequentialImpulseConstraintSolver.cpp:1878-1904)
    for (SBody& sb : s.bodies) {
        if (sb.obj < 0) continue;
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
}

// ================================================================ world step
void update_bp_aabb(Arena& a, int obj) {  // btCollisionWorld::updateSingleAabb + btRSBroadphase::setAabb
    V3 mn, mx, mn2, mx2;
    Body& b = a.body(obj);
    if (obj == OBJ_BALL) {
        ball_aabb(a, b.xf, mn, mx);
        ball_aabb(a, b.interp, mn2, mx2);
    } else {
        Car& c = a.cars[obj - OBJ_CAR0];
        car_compound_aabb(c, b.xf, mn, mx);
        car_compound_aabb(c, b.interp, mn2, mx2);
    }
    V3 th(0.02f, 0.02f, 0.02f);
    mn -= th; mx += th;
    mn2 -= th; mx2 += th;
    mn = vmin(mn, mn2);
    mx = vmax(mx, mx2);
    if (mn != b.bp_min || mx != b.bp_max) {
        int old = b.cell_idx;
        b.bp_min = mn;
        b.bp_max = mx;
        int i, j, k;
        g_grid->indices(mn, i, j, k);
        int nidx = g_grid->idx(i, j, k);
        b.cell_idx = nidx;
        if (old != nidx) {
            b.ci = i; b.cj = j; b.ck = k;
            b.cell_seq = a.cell_seq++;
        }
    }
}

void register_new_dynamic(Arena& a, Body& b, V3 mn, V3 mx) {  // createProxy for a dynamic object
    b.bp_min = mn;
    b.bp_max = mx;
    g_grid->indices(mn, b.ci, b.cj, b.ck);
    b.cell_idx = g_grid->idx(b.ci, b.cj, b.ck);
    b.cell_seq = a.cell_seq++;
}

void step_world(Arena& a) {
    float dt = a.tick_time;
    std::vector<int> dyn;  // dynamic collision objects in array order
    dyn.push_back(OBJ_BALL);
    for (size_t i = 0; i < a.cars.size(); i++) dyn.push_back(OBJ_CAR0 + (int)i);
    // applyGravity (btDiscreteDynamicsWorld.cpp:265-277)
    for (int o : dyn) {
        Body& b = a.body(o);
        if (b.is_active()) b.apply_central_force(b.gravity);
    }
    // predictUnconstraintMotion (btDiscreteDynamicsWorld.cpp:1029-1044)
    for (int o : dyn) {
        Body& b = a.body(o);
        b.lin_vel *= std::pow(1.f - b.lin_damping, dt);
        b.ang_vel *= std::pow(1.f - 0.f, dt);
        integrate_transform(b.xf, b.lin_vel, b.ang_vel, dt, b.no_rot, b.interp);
    }
    // updateAabbs
    for (int o : dyn)
        if (true) update_bp_aabb(a, o);
    // calculateOverlappingPairs (btRSBroadphase.cpp:392-468)
    std::vector<PairRec> pairs;
    auto has_pair = [&](int x, int y) {
        for (auto& p : pairs)
            if ((p.o0 == x && p.o1 == y) || (p.o0 == y && p.o1 == x)) return true;
        return false;
    };
    V3 mesh_mn, mesh_mx;
    if (a.has_arena) {
        mesh_aabb(mesh_mn, mesh_mx);
        mesh_mn -= V3(0.02f, 0.02f, 0.02f);
        mesh_mx += V3(0.02f, 0.02f, 0.02f);
    }
    std::vector<int> cell_dyn;
    for (int o : dyn) {
        Body& b = a.body(o);
        if (a.has_arena) {
            if (g_grid->mesh_cells[b.cell_idx] && aabb_overlap(b.bp_min, b.bp_max, mesh_mn, mesh_mx))
                if (!has_pair(OBJ_MESH, o)) pairs.push_back({OBJ_MESH, o});
            for (int p = 0; p < 4; p++) {
                const Plane& pl = a.planes[p];
                if (aabb_overlap(b.bp_min, b.bp_max, pl.aabb_min, pl.aabb_max))
                    if (!has_pair(OBJ_PLANE0 + p, o)) pairs.push_back({OBJ_PLANE0 + p, o});
            }
        }
        cell_dyn_list(a, b.ci, b.cj, b.ck, cell_dyn);
        if (cell_dyn.size() > 1) {
            for (int q : cell_dyn) {
                if (q == o) continue;
                Body& bq = a.body(q);
                if (aabb_overlap(b.bp_min, b.bp_max, bq.bp_min, bq.bp_max) && !has_pair(o, q))
                    pairs.push_back({std::min(o, q), std::max(o, q)});
            }
        }
    }
    // dispatchAllCollisionPairs: algorithms and manifolds in pair order
    std::vector<Manifold> mans;
    for (const PairRec& pr : pairs) {
        int o0 = pr.o0, o1 = pr.o1;
        bool act0 = a.is_static(o0) ? false : a.body(o0).is_active();
        bool act1 = a.body(o1).is_active();
        if (!act0 && !act1) continue;  // btCollisionDispatcher::needsCollision
        if (a.is_static(o0)) {
            int d = o1;
            if (d == OBJ_BALL) {
                Convex sph;
                sph.type = 1;
                sph.margin = a.ball_radius;
                Manifold m;
                m.body0 = OBJ_BALL;
                m.body1 = o0;
                m.breaking = a.ball_threshold;
                if (o0 == OBJ_MESH) convex_vs_mesh(a, m, OBJ_BALL, a.ball.xf, sph);
                else convex_vs_plane(a, m, a.ball.xf, sph, o0);
                mans.push_back(m);
            } else {
                Car& c = a.cars[d - OBJ_CAR0];
                Xf cx;
                car_child_xf(c, cx);
                Convex box;
                box.type = 0;
                box.he = c.hitbox_he;
                box.margin = c.hitbox_margin;
                Manifold m;
                m.body0 = d;
                m.body1 = o0;
                m.breaking = c.breaking_threshold;
                V3 bmn, bmx;
                car_box_aabb(c, cx, bmn, bmx);
                V3 omn, omx;
                if (o0 == OBJ_MESH) mesh_aabb(omn, omx);
                else {
                    omn = a.planes[o0 - OBJ_PLANE0].raw_min;
                    omx = a.planes[o0 - OBJ_PLANE0].raw_max;
                }
                bool ov = aabb_overlap(bmn, bmx, omn, omx);
                if (ov) {
                    if (o0 == OBJ_MESH) convex_vs_mesh(a, m, d, cx, box);
                    else convex_vs_plane(a, m, cx, box, o0);
                    mans.push_back(m);
                }
            }
        } else if (o0 == OBJ_BALL) {
            // ball (sphere) vs car (compound): child box vs sphere via GJK, manifold (car, ball)
            Car& c = a.cars[o1 - OBJ_CAR0];
            Xf cx;
            car_child_xf(c, cx);
            V3 bmn, bmx, smn, smx;
            car_box_aabb(c, cx, bmn, bmx);
            ball_aabb(a, a.ball.xf, smn, smx);
            if (aabb_overlap(bmn, bmx, smn, smx)) {
                Manifold m;
                m.body0 = o1;
                m.body1 = OBJ_BALL;
                m.breaking = std::min(c.breaking_threshold, a.ball_threshold);
                Convex box;
                box.type = 0;
                box.he = c.hitbox_he;
                box.margin = c.hitbox_margin;
                Convex sph;
                sph.type = 1;
                sph.margin = a.ball_radius;
                float md = box.margin + sph.margin + m.breaking;
                GjkOut g = gjk(box, cx, sph, a.ball.xf, md * md);
                a.counters[5]++;
                if (g.epa_needed) a.counters[3]++;
                Xf x0 = c.rb.xf, x1 = a.ball.xf;
                if (g.valid) {
                    float fr = combined_friction(a, OBJ_BALL, o1), re = combined_restitution(a, OBJ_BALL, o1);
                    // resultOut bodies are (ball, car box) while the manifold is (car, ball)
                    int idx = add_point(a, m, x0, x1, g.normal, g.point_on_b, g.dist, true, fr, re);
                    if (idx >= 0) contact_added(a, m, idx, -1);
                }
                refresh(m, x0, x1);
                mans.push_back(m);
            }
        } else {
            // car vs car: btCompoundCompoundCollisionAlgorithm (btCompoundCompoundCollisionAlgorithm.cpp:
            // 213-330) over the single box child of each car, then btBoxBoxCollisionAlgorithm
            // (btBoxBoxCollisionAlgorithm.cpp:47-72) with its own manifold
            a.counters[6]++;
            // the pair's algorithm runs with the later-added car as body 0: the manifold is
            // (higher car, lower car), which is what reproduces the reference's contacts
            int ca = o1, cb = o0;
            Car& c0 = a.cars[ca - OBJ_CAR0];
            Car& c1 = a.cars[cb - OBJ_CAR0];
            // root volumes of the compounds' child trees: child AABBs in compound space
            V3 h0 = c0.hitbox_he + V3(c0.hitbox_margin, c0.hitbox_margin, c0.hitbox_margin);
            V3 h1 = c1.hitbox_he + V3(c1.hitbox_margin, c1.hitbox_margin, c1.hitbox_margin);
            Xf l0 = xf_identity(), l1 = xf_identity();
            l0.o = c0.hitbox_off;
            l1.o = c1.hitbox_off;
            V3 amn, amx, bmn, bmx;
            transform_aabb(c0.hitbox_he, c0.hitbox_margin, l0, amn, amx);
            transform_aabb(c1.hitbox_he, c1.hitbox_margin, l1, bmn, bmx);
            Xf rel = xf_mul(xf_inverse(c0.rb.xf), c1.rb.xf);
            V3 rmn, rmx;
            transform_aabb_mm(bmn, bmx, rel, rmn, rmx);
            bool root = (amn.x <= rmx.x) && (amx.x >= rmn.x) && (amn.y <= rmx.y) && (amx.y >= rmn.y) && (amn.z <= rmx.z) &&
                        (amx.z >= rmn.z);
            if (root) {
                Xf w0, w1;
                car_child_xf(c0, w0);
                car_child_xf(c1, w1);
                V3 m0, x0v, m1, x1v;
                car_box_aabb(c0, w0, m0, x0v);
                car_box_aabb(c1, w1, m1, x1v);
                if (aabb_overlap(m0, x0v, m1, x1v)) {
                    Manifold m;
                    m.body0 = ca;
                    m.body1 = cb;
                    m.breaking = std::min(c0.breaking_threshold, c1.breaking_threshold);
                    V3 nrm;
                    BoxHit hits[4];
                    int nh = box_box(w0.o, w0.b, h0, w1.o, w1.b, h1, nrm, hits);
                    float fr = combined_friction(a, ca, cb), re = combined_restitution(a, ca, cb);
                    for (int k = 0; k < nh; k++) {
                        int idx = add_point(a, m, c0.rb.xf, c1.rb.xf, -nrm, hits[k].point, -hits[k].depth, false, fr, re);
                        if (idx >= 0) contact_added(a, m, idx, -1);
                    }
                    refresh(m, c0.rb.xf, c1.rb.xf);
                    mans.push_back(m);
                }
            }
        }
    }
    // islands (btSimulationIslandManager with STATIC_SIMULATION_ISLAND_OPTIMIZATION)
    int nd = (int)dyn.size();
    std::vector<int> uf_id(nd), uf_sz(nd, 1);
    for (int i = 0; i < nd; i++) uf_id[i] = i;
    auto find = [&](int x) { while (x != uf_id[x]) x = uf_id[x]; return x; };
    auto merges = [&](int o) { return !a.is_static(o) && !a.body(o).no_contact_response; };
    for (const PairRec& pr : pairs) {
        if (merges(pr.o0) && merges(pr.o1)) {
            int i = find(pr.o0 - OBJ_BALL), j = find(pr.o1 - OBJ_BALL);
            if (i == j) continue;
            if (uf_sz[i] < uf_sz[j]) { uf_id[i] = j; uf_sz[j] += uf_sz[i]; }
            else { uf_id[j] = i; uf_sz[i] += uf_sz[j]; }
        }
    }
    std::vector<int> tag(nd);
    for (int i = 0; i < nd; i++) tag[i] = find(i);
    auto island_of = [&](int o) { return a.is_static(o) ? -1 : tag[o - OBJ_BALL]; };
    // buildIslands: activation update per island
    {
        std::vector<int> ids(tag);
        std::sort(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        for (int id : ids) {
            bool all_sleeping = true;
            for (int i = 0; i < nd; i++) {
                if (tag[i] != id) continue;
                int st = a.body(OBJ_BALL + i).act;
                if (st == ACTIVE_TAG || st == DISABLE_DEACTIVATION) { all_sleeping = false; break; }
            }
            for (int i = 0; i < nd; i++) {
                if (tag[i] != id) continue;
                Body& b = a.body(OBJ_BALL + i);
                if (all_sleeping) {
                    if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = ISLAND_SLEEPING;
                } else if (b.act == ISLAND_SLEEPING) {
                    b.act = WANTS_DEACTIVATION;
                    b.deact_time = 0;
                }
            }
        }
    }
    std::vector<Manifold*> island_mans;
    for (Manifold& m : mans) {
        int s0 = a.is_static(m.body0) ? ISLAND_SLEEPING : a.body(m.body0).act;
        int s1 = a.is_static(m.body1) ? ISLAND_SLEEPING : a.body(m.body1).act;
        if (s0 != ISLAND_SLEEPING || s1 != ISLAND_SLEEPING) {
            bool r0 = a.is_static(m.body0) ? true : !a.body(m.body0).no_contact_response;
            bool r1 = a.is_static(m.body1) ? true : !a.body(m.body1).no_contact_response;
            bool resp = r0 && r1 && (!a.is_static(m.body0) || !a.is_static(m.body1));
            if (resp) {
                m.island = island_of(m.body0) >= 0 ? island_of(m.body0) : island_of(m.body1);
                island_mans.push_back(&m);
            }
        }
    }
    if (island_mans.size() > 1)
        bt_quicksort(island_mans, [](Manifold* l, Manifold* r) { return l->island < r->island; }, 0,
                     (int)island_mans.size() - 1);
    // processIslands: bodies and manifolds of awake islands, solved as one batch
    std::vector<int> bodies;
    std::vector<Manifold*> solve_mans;
    {
        std::vector<int> ids(tag);
        std::sort(ids.begin(), ids.end());
        ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
        for (int id : ids) {
            bool sleeping = true;
            std::vector<int> ib;
            for (int i = 0; i < nd; i++)
                if (tag[i] == id) {
                    ib.push_back(OBJ_BALL + i);
                    if (a.body(OBJ_BALL + i).is_active()) sleeping = false;
                }
            if (sleeping) continue;
            for (int o : ib) bodies.push_back(o);
            for (Manifold* m : island_mans)
                if (m->island == id) solve_mans.push_back(m);
        }
    }
    a.solver_dt = dt;
    if (!bodies.empty()) solve(a, bodies, solve_mans, dt);
    // integrateTransforms (btDiscreteDynamicsWorld.cpp:889-991)
    for (int o : dyn) {
        Body& b = a.body(o);
        if (b.is_active()) {
            Xf nt;
            integrate_transform(b.xf, b.lin_vel, b.ang_vel, dt, b.no_rot, nt);
            b.interp = nt;
            b.xf = nt;
            b.update_inertia();
        }
    }
    // updateActivationState (btDiscreteDynamicsWorld.cpp:516-551)
    for (int o : dyn) {
        Body& b = a.body(o);
        if (b.act == ISLAND_SLEEPING || b.act == DISABLE_DEACTIVATION) {
        } else if (len2(b.lin_vel) < 0.8f * 0.8f && len2(b.ang_vel) < 1.f * 1.f) {
            b.deact_time += dt;
        } else {
            b.deact_time = 0;
            if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = 0;
        }
        bool wants = false;
        if (b.act != DISABLE_DEACTIVATION) {
            if (b.act == ISLAND_SLEEPING || b.act == WANTS_DEACTIVATION) wants = true;
            else if (b.deact_time > 2.0f) wants = true;
        }
        if (wants) {
            if (b.act == ACTIVE_TAG) b.act = WANTS_DEACTIVATION;
            if (b.act == ISLAND_SLEEPING) { b.ang_vel = V3(0, 0, 0); b.lin_vel = V3(0, 0, 0); }
        } else {
            if (b.act != DISABLE_DEACTIVATION && b.act != DISABLE_SIMULATION) b.act = ACTIVE_TAG;
        }
    }
    // clearForces
    for (int o : dyn) {
        Body& b = a.body(o);
        b.total_force = V3(0, 0, 0);
        b.total_torque = V3(0, 0, 0);
    }
}

bool ball_scored(Arena& a) {  // Arena::IsBallScored soccar (Arena.cpp:893-901)
    float y = a.ball.xf.o.y * BT_TO_UU;
    return std::fabs(y) > (RL::SOCCAR_GOAL_SCORE_BASE_THRESHOLD_Y + RL::BALL_COLLISION_RADIUS_SOCCAR);
}

void pad_check(Arena& a, Pad& p, int ci) {  // BoostPad::_CheckCollide (BoostPad.cpp:62-86)
    Car& c = a.cars[ci];
    V3 cp = c.rb.xf.o;
    bool col = false;
    if (p.prev_locked_id == c.id) {
        V3 mn, mx;
        car_compound_aabb(c, c.rb.xf, mn, mx);
        // Vec operator> / < compare all three components
        bool gt = (p.box_max.x > mn.x) && (p.box_max.y > mn.y) && (p.box_max.z > mn.z);
        bool lt = (p.box_min.x < mx.x) && (p.box_min.y < mx.y) && (p.box_min.z < mx.z);
        col = gt && lt;
    } else {
        float rad = (p.big ? RL::Pads::CYL_RAD_BIG : RL::Pads::CYL_RAD_SMALL) * UU_TO_BT;
        float dx = cp.x - p.pos_bt.x, dy = cp.y - p.pos_bt.y;
        if (dx * dx + dy * dy < rad * rad) col = std::fabs(cp.z - p.pos_bt.z) < (RL::Pads::CYL_HEIGHT * UU_TO_BT);
    }
    if (col) p.cur_locked = ci;
}

void grid_check(Arena& a, int ci) {  // BoostPadGrid::CheckCollision (BoostPadGrid.cpp:5-25)
    Car& c = a.cars[ci];
    if (c.st.is_demoed || c.st.boost >= RL::BOOST_MAX) return;
    V3 cp = c.rb.xf.o * BT_TO_UU;
    const float EXT_Z = RL::Pads::CYL_HEIGHT + 250.f;
    if (cp.z > EXT_Z) return;
    const int CX = 8, CY = 10, SX = (int)(4096.f / (CX / 2)), SY = (int)(5120.f / (CY / 2));
    int ix = (int)(cp.x / SX + (CX / 2));
    int iy = (int)(cp.y / SY + (CY / 2));
    for (int i = std::max(ix - 1, 0); i <= std::min(ix + 1, CX - 1); i++)
        for (int j = std::max(iy - 1, 0); j <= std::min(iy + 1, CY - 1); j++) {
            for (int k = 0; k < a.npads; k++) {
                const Pad& p = a.pads[k];
                int px = (int)(p.pos_uu.x / SX + (CX / 2));
                int py = (int)(p.pos_uu.y / SY + (CY / 2));
                if (px == i && py == j) pad_check(a, a.pads[k], ci);
            }
        }
}

void arena_step(Arena& a) {  // Arena::Step (Arena.cpp:689-756)
    Body& ball = a.ball;
    if (len2(ball.lin_vel) == 0 && len2(ball.ang_vel) == 0) {
        if (ball.act != DISABLE_DEACTIVATION && ball.act != DISABLE_SIMULATION) ball.act = ISLAND_SLEEPING;
    } else {
        if (ball.act != DISABLE_DEACTIVATION && ball.act != DISABLE_SIMULATION) ball.act = ACTIVE_TAG;
    }
    bool ball_only = a.cars.empty();
    for (int ci : a.order) car_pre_tick(a, a.cars[ci]);
    if (a.has_arena && !ball_only)
        for (int i = 0; i < a.npads; i++) {  // BoostPad::_PreTickUpdate (BoostPad.cpp:51-60)
            Pad& p = a.pads[i];
            if (p.cooldown > 0) p.cooldown = rs_max(p.cooldown - a.tick_time, 0);
            p.active = (p.cooldown == 0);
            p.cur_locked = -1;
        }
    step_world(a);
    for (int ci : a.order) {
        car_post_tick(a, a.cars[ci]);
        car_finish_physics(a.cars[ci]);
        if (a.has_arena) grid_check(a, ci);
    }
    if (a.has_arena && !ball_only)
        for (int i = 0; i < a.npads; i++) {  // BoostPad::_PostTickUpdate (BoostPad.cpp:88-105)
            Pad& p = a.pads[i];
            uint32_t locked = 0;
            if (p.cur_locked >= 0) {
                Car& c = a.cars[p.cur_locked];
                locked = c.id;
                if (p.active) {
                    float add = p.big ? RL::Pads::BOOST_AMOUNT_BIG : RL::Pads::BOOST_AMOUNT_SMALL;
                    c.st.boost = rs_min(c.st.boost + add, RL::BOOST_MAX);
                    p.active = false;
                    p.cooldown = p.big ? RL::Pads::COOLDOWN_BIG : RL::Pads::COOLDOWN_SMALL;
                }
            }
            p.prev_locked_id = locked;
        }
    {  // Ball::_FinishPhysicsTick (Ball.cpp:117-143)
        if (!is_zero(a.ball_cache)) {
            ball.lin_vel += a.ball_cache;
            a.ball_cache = V3(0, 0, 0);
        }
        V3 v = ball.lin_vel, w = ball.ang_vel;
        float ms = RL::BALL_MAX_SPEED * UU_TO_BT;
        if (len2(v) > ms * ms) v = normalized(v) * ms;
        if (len2(w) > (RL::BALL_MAX_ANG_SPEED * RL::BALL_MAX_ANG_SPEED)) w = normalized(w) * RL::BALL_MAX_ANG_SPEED;
        ball.lin_vel = v;
        ball.ang_vel = w;
        a.ball_ticks++;
    }
    if (a.has_arena && ball_scored(a)) {
        uint32_t team = (-(a.ball.xf.o.y) < 0) ? 0 : 1;  // RS_TEAM_FROM_Y(-y)
        a.events.push_back({RSG_EVENT_GOAL, a.tick_count, team, 0, 0});
    }
    a.tick_count++;
}

Car* find_car(Arena& a, uint32_t id) {
    for (Car& c : a.cars)
        if (c.id == id) return &c;
    return nullptr;
}

}  // namespace

extern "C" {

int rsora_init(const uint8_t* cmf, uint64_t len) {
    if (g_inited) return 0;
    auto m = std::make_unique<Mesh>();
    if (!m->load(cmf, len)) return -1;
    g_mesh = std::move(m);
    g_grid = std::make_unique<Grid>();
    V3 mn, mx;
    mesh_aabb(mn, mx);
    g_grid->register_mesh(*g_mesh, mn - V3(0.02f, 0.02f, 0.02f), mx + V3(0.02f, 0.02f, 0.02f));
    g_inited = true;
    return 0;
}

void* rsora_arena_create(int game_mode, float tick_rate) {
    if (game_mode != RSG_GAMEMODE_THE_VOID && !g_inited) return nullptr;
    if (!g_grid) g_grid = std::make_unique<Grid>();
    Arena* a = new Arena();
    setup_arena(*a, game_mode, tick_rate);
    // the ball proxy is created before any car (Arena.cpp:491-496)
    V3 mn, mx;
    ball_aabb(*a, a->ball.xf, mn, mx);
    register_new_dynamic(*a, a->ball, mn - V3(0.02f, 0.02f, 0.02f), mx + V3(0.02f, 0.02f, 0.02f));
    return a;
}

void rsora_arena_destroy(void* h) { delete (Arena*)h; }

int rsora_preset(int preset, rsg_car_config* out) {
    if (preset < 0 || preset > 5) return -1;
    *out = preset_config(preset);
    return 0;
}

uint32_t rsora_add_car(void* h, int team, int preset) {
    Arena& a = *(Arena*)h;
    Car c;
    c.id = ++a.last_car_id;
    c.team = team;
    c.cfg = preset_config(preset);
    std::memset(&c.controls, 0, sizeof(c.controls));
    std::memset(&c.st, 0, sizeof(c.st));
    setup_car(a, c);
    c.st.boost = RL::BOOST_SPAWN_AMOUNT;
    car_respawn(c, 0, RL::BOOST_SPAWN_AMOUNT);
    a.cars.push_back(c);
    Car& cr = a.cars.back();
    cr.obj = OBJ_CAR0 + (int)a.cars.size() - 1;
    a.order.push_back((int)a.cars.size() - 1);
    // createProxy at the AddCar-time transform (identity; the respawn SetState does not touch the broadphase)
    V3 mn, mx;
    Xf ident = xf_identity();
    car_compound_aabb(cr, ident, mn, mx);
    register_new_dynamic(a, cr.rb, mn, mx);
    return cr.id;
}

int rsora_car_order(void* h, uint32_t* out, uint32_t cap) {
    Arena& a = *(Arena*)h;
    uint32_t n = 0;
    for (int ci : a.order) {
        if (n < cap) out[n] = a.cars[ci].id;
        n++;
    }
    return (int)n;
}

int rsora_set_car_order(void* h, const uint32_t* ids, uint32_t n) {
    Arena& a = *(Arena*)h;
    if (n != a.cars.size()) return -1;
    std::vector<int> o;
    for (uint32_t i = 0; i < n; i++) {
        int f = -1;
        for (size_t k = 0; k < a.cars.size(); k++)
            if (a.cars[k].id == ids[i]) f = (int)k;
        if (f < 0) return -1;
        o.push_back(f);
    }
    a.order = o;
    return 0;
}

int rsora_set_controls(void* h, uint32_t id, const rsg_car_controls* c) {
    Car* car = find_car(*(Arena*)h, id);
    if (!car) return -1;
    car->controls = *c;
    return 0;
}

int rsora_get_car(void* h, uint32_t id, rsg_car_state* out) {
    Car* car = find_car(*(Arena*)h, id);
    if (!car) return -1;
    car_refresh_state(*car);
    *out = car->st;
    return 0;
}

int rsora_set_car(void* h, uint32_t id, const rsg_car_state* s) {
    Car* car = find_car(*(Arena*)h, id);
    if (!car) return -1;
    car_set_state(*car, *s);
    return 0;
}

int rsora_get_ball(void* h, rsg_ball_state* out) {
    get_ball_state(*(Arena*)h, *out);
    return 0;
}

int rsora_set_ball(void* h, const rsg_ball_state* in) {
    set_ball_state(*(Arena*)h, *in);
    return 0;
}

int rsora_num_pads(void* h) { return ((Arena*)h)->npads; }

int rsora_get_pad(void* h, int i, rsg_pad_state* out) {
    Arena& a = *(Arena*)h;
    if (i < 0 || i >= a.npads) return -1;
    std::memset(out, 0, sizeof(*out));
    out->is_active = a.pads[i].active;
    out->cooldown = a.pads[i].cooldown;
    out->cur_locked_car_id = a.pads[i].cur_locked >= 0 ? a.cars[a.pads[i].cur_locked].id : 0;
    out->prev_locked_car_id = a.pads[i].prev_locked_id;
    return 0;
}

int rsora_set_pad(void* h, int i, const rsg_pad_state* in) {
    Arena& a = *(Arena*)h;
    if (i < 0 || i >= a.npads) return -1;
    a.pads[i].active = in->is_active;
    a.pads[i].cooldown = in->cooldown;
    a.pads[i].cur_locked = -1;
    a.pads[i].prev_locked_id = in->prev_locked_car_id;
    return 0;
}

int rsora_pad_config(void* h, int i, rsg_vec3* pos, int* is_big) {
    Arena& a = *(Arena*)h;
    if (i < 0 || i >= a.npads) return -1;
    *pos = P(a.pads[i].pos_uu);
    *is_big = a.pads[i].big;
    return 0;
}

uint64_t rsora_get_tick(void* h) { return ((Arena*)h)->tick_count; }
void rsora_set_tick(void* h, uint64_t t) { ((Arena*)h)->tick_count = t; }

int rsora_step(void* h, int ticks) {
    Arena& a = *(Arena*)h;
    for (int i = 0; i < ticks; i++) arena_step(a);
    return 0;
}

// Steps `ticks` ticks, setting the controls of car k (AddCar order) from
// controls[t * ncars + k] before tick t (timing helper, no per-tick caller round trip).
int rsora_run(void* h, const rsg_car_controls* controls, int ncars, int ticks) {
    Arena& a = *(Arena*)h;
    if (ncars != (int)a.cars.size()) return -1;
    for (int t = 0; t < ticks; t++) {
        for (int k = 0; k < ncars; k++) a.cars[k].controls = controls[(size_t)t * ncars + k];
        arena_step(a);
    }
    return 0;
}

int rsora_is_scored(void* h) { return ball_scored(*(Arena*)h) ? 1 : 0; }

int rsora_pop_events(void* h, uint64_t* out, int cap) {
    Arena& a = *(Arena*)h;
    int n = 0;
    for (auto& e : a.events) {
        if (e.kind == RSG_EVENT_BALL_HIT) continue;  // the reference driver has no ball-hit event
        if (n >= cap) break;
        out[n * 5 + 0] = e.kind;
        out[n * 5 + 1] = e.tick;
        out[n * 5 + 2] = e.a;
        out[n * 5 + 3] = e.b;
        out[n * 5 + 4] = e.flag;
        n++;
    }
    a.events.clear();
    return n;
}

int rsora_get_wheel_internals(void* h, uint32_t id, float* out8) {
    Car* car = find_car(*(Arena*)h, id);
    if (!car) return -1;
    for (int i = 0; i < 4; i++) {
        out8[i] = car->w[i].steer;
        out8[4 + i] = car->w[i].extra_pushback;
    }
    return 0;
}

int rsora_wheel_debug(void* h, uint32_t id, float* out) {
    Car* car = find_car(*(Arena*)h, id);
    if (!car) return -1;
    for (int i = 0; i < 4; i++) {
        const Wheel& w = car->w[i];
        float* o = out + i * 16;
        o[0] = w.contact_point.x; o[1] = w.contact_point.y; o[2] = w.contact_point.z;
        o[3] = w.contact_normal.x; o[4] = w.contact_normal.y; o[5] = w.contact_normal.z;
        o[6] = w.susp_len; o[7] = w.susp_rel_vel; o[8] = w.clipped_inv_dot;
        o[9] = w.impulse.x; o[10] = w.impulse.y; o[11] = w.impulse.z;
        o[12] = w.lat_fric; o[13] = w.long_fric; o[14] = w.hard_point.z;
        o[15] = w.ground < 0 ? 0.f : (w.ground < OBJ_BALL ? 1.f : 2.f);
    }
    return 0;
}

// The suspension ray of one wheel at the current state, traced object by object (test aid): writes
// from (3), to (3), then per hit candidate (kind 0 mesh triangle / 1 plane, index, accepted, fraction)
// up to `cap` candidates; returns the number of candidates.
int rsora_debug_wheel_ray(void* h, uint32_t id, int wheel, float* out, int cap) {
    Arena& a = *(Arena*)h;
    Car* car = find_car(a, id);
    if (!car || wheel < 0 || wheel > 3) return -1;
    Wheel w = car->w[wheel];
    wheel_transforms_ws(*car, w);
    float travel = w.travel_cm / 100;
    float ray_len = w.rest_len + travel + w.radius - RL::BTV::SUSPENSION_SUBTRACTION;
    V3 src = w.hard_point, dst = src + (w.dir_ws * ray_len);
    out[0] = src.x; out[1] = src.y; out[2] = src.z; out[3] = dst.x; out[4] = dst.y; out[5] = dst.z;
    int n = 0;
    float frac = 1.f;
    const Mesh& m = *g_mesh;
    m.query_ray(src, dst, [&](int t) {
        V3 tv[3];
        m.tri_verts(t, tv);
        V3 nn;
        float f0 = frac;
        bool ok = ray_triangle(src, dst, tv, frac, nn);
        if (n < cap) { float* o = out + 6 + 4 * n; o[0] = 0; o[1] = (float)t; o[2] = ok; o[3] = ok ? frac : f0; }
        n++;
    });
    for (int p = 0; p < 4; p++) {
        V3 nn;
        bool ok = ray_plane(a.planes[p], src, dst, frac, nn);
        if (n < cap) { float* o = out + 6 + 4 * n; o[0] = 1; o[1] = (float)p; o[2] = ok; o[3] = frac; }
        n++;
    }
    int ci, cj, ck;
    g_grid->indices(src, ci, cj, ck);
    std::vector<int> dyn;
    cell_dyn_list(a, ci, cj, ck, dyn);
    for (int o : dyn) {
        if (o == car->obj) continue;
        V3 nn;
        bool ok;
        if (o == OBJ_BALL) {
            ok = ray_cast_sphere(src, dst, a.ball.xf, a.ball_radius, frac, nn);
        } else {
            Car& c = a.cars[o - OBJ_CAR0];
            Xf bx = c.rb.xf;
            bx.o = xf_apply(c.rb.xf, c.hitbox_off);
            V3 he = c.hitbox_he + V3(c.hitbox_margin, c.hitbox_margin, c.hitbox_margin);
            ok = ray_cast_box(src, dst, bx, he, frac, nn);
        }
        if (n < cap) { float* q = out + 6 + 4 * n; q[0] = 2; q[1] = (float)o; q[2] = ok; q[3] = frac; }
        n++;
    }
    return n;
}

int rsora_body_debug(void* h, uint32_t id, float* out) {
    Car* car = find_car(*(Arena*)h, id);
    if (!car) return -1;
    out[0] = car->rb.inv_inertia_local.x; out[1] = car->rb.inv_inertia_local.y; out[2] = car->rb.inv_inertia_local.z;
    out[3] = car->rb.inv_mass;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) out[4 + i * 3 + j] = car->rb.inv_inertia_world.r[i][j];
    out[13] = car->hitbox_he.x; out[14] = car->hitbox_he.y; out[15] = car->hitbox_he.z; out[16] = car->hitbox_margin;
    return 0;
}

int rsora_get_counters(void* h, uint64_t* out, int cap) {
    Arena& a = *(Arena*)h;
    int n = std::min(cap, 16);
    for (int i = 0; i < n; i++) out[i] = a.counters[i];
    return n;
}

}  // extern "C"
