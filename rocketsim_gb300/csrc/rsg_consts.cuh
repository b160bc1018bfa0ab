// rsg_consts.cuh -- Rocket League constants, curves and car presets used by the tick.
//
// Values are RocketSim's (src/RLConst.h:9-503, src/Sim/Car/CarConfig/CarConfig.cpp:20-99,
// src/Sim/MutatorConfig/MutatorConfig.h defaults); they have to be the same
// numbers for the simulation to agree, so the table is restated here as data.
#pragma once
#include "rsg_math.cuh"

namespace rsg {
namespace RL {
constexpr float UU_TO_BT = 1.f / 50.f;
constexpr float BT_TO_UU = 50.f;
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
constexpr float RECHARGE_BOOST_PER_SECOND = 10, RECHARGE_BOOST_DELAY = 0.25f;
constexpr float BOOST_ACCEL_GROUND = 2975 / 3.f, BOOST_ACCEL_AIR = 3175 / 3.f, BOOST_SPAWN_AMOUNT = BOOST_MAX / 3;
constexpr float CAR_MAX_ANG_SPEED = 5.5f;
constexpr float SUPERSONIC_START_SPEED = 2200.f, SUPERSONIC_MAINTAIN_MIN_SPEED = SUPERSONIC_START_SPEED - 100.f;
constexpr float SUPERSONIC_MAINTAIN_MAX_TIME = 1.f;
constexpr float ARENA_EXTENT_Y = 5120;
// Heatseeker (src/RLConst.h:168-190)
namespace HS {
constexpr float INITIAL_TARGET_SPEED = 2900, TARGET_SPEED_INCREMENT = 85, MIN_SPEEDUP_INTERVAL = 1;
constexpr float TARGET_Y = 5120, TARGET_Z = 320, HORIZONTAL_BLEND = 1.45f, VERTICAL_BLEND = 0.78f,
                SPEED_BLEND = 0.3f;
constexpr float MAX_TURN_PITCH = (float)(7000 * 3.14159265358979323846 / (1 << 15)), MAX_SPEED = 4600;
constexpr float WALL_BOUNCE_CHANGE_Y_THRESH = 300, WALL_BOUNCE_CHANGE_Y_NORMAL = 0.5f,
                WALL_BOUNCE_FORCE_SCALE = 1 / 3.f, WALL_BOUNCE_UP_FRAC = 0.3f;
constexpr float BALL_START_POS[3] = {-1000, -2220, 92.75f}, BALL_START_VEL[3] = {0, -65, 650};
}  // namespace HS
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
constexpr float CAR_RESPAWN_Z = 36.f, CAR_SPAWN_REST_Z = 17.f;
constexpr float BUMP_COOLDOWN_TIME = 0.25f, BUMP_MIN_FORWARD_DIST = 64.5f, DEMO_RESPAWN_TIME = 3.f;
constexpr float AIR_TORQUE_X = 130, AIR_TORQUE_Y = 95, AIR_TORQUE_Z = 400;
constexpr float AIR_DAMP_X = 30, AIR_DAMP_Y = 20, AIR_DAMP_Z = 50;
constexpr float SUSPENSION_FORCE_SCALE_FRONT = 36.f - (1.f / 4.f);
constexpr float SUSPENSION_FORCE_SCALE_BACK = 54.f + (1.f / 4.f) + (1.5f / 100.f);
constexpr float SUSPENSION_STIFFNESS = 500.f, WHEELS_DAMPING_COMPRESSION = 25.f;
constexpr float WHEELS_DAMPING_RELAXATION = 40.f, MAX_SUSPENSION_TRAVEL = 12.f, SUSPENSION_SUBTRACTION = 0.05f;
constexpr float PAD_CYL_HEIGHT = 95, PAD_CYL_RAD_BIG = 208, PAD_CYL_RAD_SMALL = 144, PAD_BOX_HEIGHT = 64;
constexpr float PAD_BOX_RAD_BIG = 160, PAD_BOX_RAD_SMALL = 120, PAD_COOLDOWN_BIG = 10, PAD_COOLDOWN_SMALL = 4;
constexpr float PAD_BOOST_BIG = 100, PAD_BOOST_SMALL = 12;
}  // namespace RL

// Boost pad locations (RLConst.h:265-305): 6 big pads first, then 28 small ones
// (Arena.cpp:514-531).  Stored as x, y, z in uu.
#define RSG_PAD_LOCS_INIT                                                                                   \
    {{-3584.f, 0.f, 73.f}, {3584.f, 0.f, 73.f}, {-3072.f, 4096.f, 73.f}, {3072.f, 4096.f, 73.f},                    \
     {-3072.f, -4096.f, 73.f}, {3072.f, -4096.f, 73.f},                                                              \
     {0.f, -4240.f, 70.f}, {-1792.f, -4184.f, 70.f}, {1792.f, -4184.f, 70.f}, {-940.f, -3308.f, 70.f},              \
     {940.f, -3308.f, 70.f}, {0.f, -2816.f, 70.f}, {-3584.f, -2484.f, 70.f}, {3584.f, -2484.f, 70.f},               \
     {-1788.f, -2300.f, 70.f}, {1788.f, -2300.f, 70.f}, {-2048.f, -1036.f, 70.f}, {0.f, -1024.f, 70.f},             \
     {2048.f, -1036.f, 70.f}, {-1024.f, 0.f, 70.f}, {1024.f, 0.f, 70.f}, {-2048.f, 1036.f, 70.f},                   \
     {0.f, 1024.f, 70.f}, {2048.f, 1036.f, 70.f}, {-1788.f, 2300.f, 70.f}, {1788.f, 2300.f, 70.f},                  \
     {-3584.f, 2484.f, 70.f}, {3584.f, 2484.f, 70.f}, {0.f, 2816.f, 70.f}, {-940.f, 3308.f, 70.f},                  \
     {940.f, 3308.f, 70.f}, {-1792.f, 4184.f, 70.f}, {1792.f, 4184.f, 70.f}, {0.f, 4240.f, 70.f}}
constexpr float PAD_LOCS[34][3] = RSG_PAD_LOCS_INIT;

// Respawn locations for the blue team (RLConst.h:340-346); yaw is pi/2 for all.
constexpr float RESPAWN_LOCS[4][2] = {{-2304, -4608}, {-2688, -4608}, {2304, -4608}, {2688, -4608}};

// LinearPieceCurve (src/Math/Math.cpp:5-35)
struct Curve {
    int n;
    float x[6], y[6];
};
// LinearPieceCurve::GetOutput: the first point above `in` and a linear interpolation from the
// point before it.  The segment is selected without early returns so that threads evaluating
// different segments share one interpolation.
RSG_HD float curve_eval(const Curve& c, float in, float def = 1) {
    const int n = c.n;
    if (n == 0) return def;
    if (in <= c.x[0]) return c.y[0];
    float xa = 0, xb = 0, ya = 0, yb = 0;
    bool found = false;
#pragma unroll
    for (int i = 1; i < 6; i++) {
        if (!found && i < n && c.x[i] > in) {
            xa = c.x[i - 1]; xb = c.x[i]; ya = c.y[i - 1]; yb = c.y[i];
            found = true;
        }
    }
    if (!found) return c.y[n - 1];
    float range = xb - xa;
    float diff = yb - ya;
    float f = (in - xa) / range;
    return ya + diff * f;
}

// Curve table (RLConst.h:388-503)
enum CurveId {
    CV_STEER = 0, CV_STEER_3W, CV_POWERSLIDE_STEER, CV_DRIVE_TORQUE, CV_NON_STICKY, CV_LAT_FRIC, CV_LAT_FRIC_3W,
    CV_LONG_FRIC, CV_HB_LAT, CV_HB_LONG, CV_BALL_EXTRA, CV_BUMP_GROUND, CV_BUMP_AIR, CV_BUMP_UP, CV_COUNT
};
#define RSG_CURVES_INIT \
    { \
    {6, {0, 500, 1000, 1500, 1750, 3000}, {0.53356f, 0.31930f, 0.18203f, 0.10570f, 0.08507f, 0.03454f}}, \
    {2, {0, 2300}, {0.342473f, 0.034837f}}, \
    {2, {0, 2500}, {0.39235f, 0.12610f}}, \
    {3, {0, 1400, 1410}, {1.0f, 0.1f, 0.0f}}, \
    {3, {0, 0.7075f, 1}, {0.1f, 0.5f, 1.0f}}, \
    {2, {0, 1}, {1.0f, 0.2f}}, \
    {2, {0, 1}, {0.30f, 0.25f}}, \
    {0, {}, {}}, \
    {1, {0}, {0.1f}}, \
    {2, {0, 1}, {0.5f, 0.9f}}, \
    {4, {0, 500.f, 2300.f, 4600.f}, {0.65f, 0.65f, 0.55f, 0.30f}}, \
    {3, {0.f, 1400.f, 2200.f}, {(5.f / 6.f), 1100.f, 1530.f}}, \
    {3, {0.f, 1400.f, 2200.f}, {(5.f / 6.f), 1390.f, 1945.f}}, \
    {3, {0.f, 1400.f, 2200.f}, {(2.f / 6.f), 278.f, 417.f}}, \
    }
constexpr Curve CURVES_INIT[CV_COUNT] = RSG_CURVES_INIT;

// Car hitbox presets (CarConfig.cpp:20-82): size, offset, front/back radius,
// front/back suspension rest, front/back wheel offsets
struct PresetData {
    float size[3], off[3], frad, brad, fsus, bsus, fwo[3], bwo[3];
};
constexpr PresetData PRESETS[6] = {
    {{120.507f, 86.6994f, 38.6591f}, {13.8757f, 0, 20.755f}, 12.50f, 15.00f, 38.755f, 37.055f, {51.25f, 25.90f, 20.755f}, {-33.75f, 29.50f, 20.755f}},
    {{130.427f, 85.7799f, 33.8f}, {9.f, 0, 15.75f}, 12.00f, 13.50f, 33.95f, 33.85f, {50.30f, 31.10f, 15.75f}, {-34.75f, 33.00f, 15.75f}},
    {{131.32f, 87.1704f, 31.8944f}, {9.00857f, 0, 12.0942f}, 12.50f, 17.00f, 31.9242f, 27.9242f, {49.97f, 27.80f, 12.0942f}, {-35.43f, 20.28f, 12.0942f}},
    {{133.992f, 83.021f, 32.8f}, {12.5f, 0, 11.75f}, 13.50f, 15.00f, 29.7f, 29.666f, {51.50f, 26.67f, 11.75f}, {-35.75f, 35.00f, 11.75f}},
    {{129.519f, 84.6879f, 36.6591f}, {13.8757f, 0, 20.755f}, 12.50f, 15.00f, 38.755f, 37.055f, {51.25f, 25.90f, 20.755f}, {-34.00f, 29.50f, 20.755f}},
    {{123.22f, 79.2103f, 44.1591f}, {11.3757f, 0, 21.505f}, 15.00f, 15.00f, 39.505f, 39.105f, {51.25f, 25.90f, 21.505f}, {-33.75f, 29.50f, 21.505f}},
};

}  // namespace rsg
