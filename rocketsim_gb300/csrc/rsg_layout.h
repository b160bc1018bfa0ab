// rsg_layout.h -- layout of a batch of arenas in device memory.
//
// Each arena's persistent state is one record of 32-bit words (ball, boost
// pads, then one fixed-size block per car slot), records stored back to back.
// One warp advances one arena and moves its record with contiguous loads and
// stores.  A second, small array holds per-arena scalars field-major
// ([field][arena]) so that the host can read one field of every arena (event
// counts, error flags) with a single copy.  Positions and velocities are kept
// in Bullet units (uu / 50) as the reference keeps them inside btRigidBody.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define RSG_LAYOUT_FN __host__ __device__ constexpr
#else
#define RSG_LAYOUT_FN constexpr
#endif

namespace rsg {

// ---- per-car float fields
enum CarF : int {
    CF_POS = 0,          // 3: rigid body origin
    CF_BASIS = 3,        // 9: rigid body basis rows
    CF_VEL = 12,         // 3
    CF_ANG = 15,         // 3
    CF_ROT = 18,         // 9: CarState::rotMat (rows of the basis copied at the last post-tick)
    CF_STEER = 27,       // front wheel steer angle of the last tick (btWheelInfoRL::m_steerAngle)
    CF_PUSHBACK = 28,    // 4: btWheelInfoRL::m_extraPushback
    CF_LATF = 32,        // 4: m_latFriction
    CF_LONGF = 36,       // 4: m_longFriction
    CF_ENGINE = 40,      // m_engineForce (same on all wheels)
    CF_BRAKE = 41,       // m_brake
    CF_FLIP_REL = 42,    // 3
    CF_JUMP_TIME = 45,
    CF_FLIP_TIME = 46,
    CF_AIR_TIME = 47,
    CF_AIR_TIME_SJ = 48,
    CF_BOOST = 49,
    CF_TIME_SINCE_BOOST = 50,
    CF_BOOSTING_TIME = 51,
    CF_SUPERSONIC_TIME = 52,
    CF_HANDBRAKE = 53,
    CF_AUTOFLIP_TIMER = 54,
    CF_AUTOFLIP_SCALE = 55,
    CF_WC_NORMAL = 56,   // 3
    CF_CC_COOLDOWN = 59,
    CF_DEMO_TIMER = 60,
    CF_BHI_REL = 61,     // 3
    CF_BHI_BALLPOS = 64, // 3
    CF_BHI_EXTRA = 67,   // 3
    CF_CTRL = 70,        // 5: throttle steer pitch yaw roll
    CF_LAST_CTRL = 75,   // 5
    CF_VEL_CACHE = 80,   // 3: bump velocity not yet applied (Car::_velocityImpulseCache)
    CF_COUNT = 83
};

// ---- per-car u32 fields
enum CarFlag : uint32_t {
    F_PRESENT = 1u << 0,
    F_ON_GROUND = 1u << 1,
    F_WHEEL0 = 1u << 2,  // 4 bits
    F_HAS_JUMPED = 1u << 6,
    F_HAS_DJ = 1u << 7,
    F_HAS_FLIPPED = 1u << 8,
    F_FLIPPING = 1u << 9,
    F_JUMPING = 1u << 10,
    F_BOOSTING = 1u << 11,
    F_SUPERSONIC = 1u << 12,
    F_AUTOFLIPPING = 1u << 13,
    F_WC_CONTACT = 1u << 14,
    F_DEMOED = 1u << 15,
    F_BHI_VALID = 1u << 16,
    F_CTRL_JUMP = 1u << 17,
    F_CTRL_BOOST = 1u << 18,
    F_CTRL_HB = 1u << 19,
    F_LAST_JUMP = 1u << 20,
    F_LAST_BOOST = 1u << 21,
    F_LAST_HB = 1u << 22,
    F_TEAM_ORANGE = 1u << 23,
    F_NO_RESPONSE = 1u << 24,  // CF_NO_CONTACT_RESPONSE of the rigid body (set at each pre-tick)
};
enum CarU : int {
    CU_FLAGS = 0,
    CU_ID = 1,
    CU_CC_OTHER = 2,     // carContact.otherCarID
    CU_CFG = 3,          // car config table index
    CU_CELL = 4,         // broadphase cell (i | j << 8 | k << 16), 0xffffffff if none
    CU_CELL_SEQ = 5,     // order of the last cell change (cell handle list order)
    CU_BHI_HIT_LO = 6,   // ballHitInfo.tickCountWhenHit
    CU_BHI_HIT_HI = 7,
    CU_BHI_EXTRA_LO = 8, // ballHitInfo.tickCountWhenExtraImpulseApplied
    CU_BHI_EXTRA_HI = 9,
    CU_TICKS_LO = 10,    // tickCountSinceUpdate
    CU_TICKS_HI = 11,
    CU_COUNT = 12
};

// ---- ball (per arena)
// BF_HS_*: BallState::HeatseekerInfo (src/Sim/Ball/Ball.h:24-32): yTargetDir, curTargetSpeed, timeSinceHit
enum BallF : int { BF_POS = 0, BF_BASIS = 3, BF_VEL = 12, BF_ANG = 15, BF_HS_DIR = 18, BF_HS_SPEED = 19, BF_HS_TIME = 20,
                   BF_COUNT = 21 };
enum BallU : int { BU_CELL = 0, BU_CELL_SEQ = 1, BU_TICKS_LO = 2, BU_TICKS_HI = 3, BU_COUNT = 4 };

// ---- pads (per arena and pad)
enum PadF : int { PF_COOLDOWN = 0, PF_COUNT = 1 };
enum PadU : int { PU_ACTIVE = 0, PU_PREV_LOCKED = 1, PU_CUR_LOCKED = 2 /* car slot + 1, 0 none */, PU_COUNT = 3 };

// ---- arena scalars
enum ArenaU : int {
    AU_TICK_LO = 0,
    AU_TICK_HI = 1,
    AU_NCARS = 2,
    AU_ORDER = 3,        // 8 slots x 4 bits: per-car update order (slot indices)
    AU_SEQ = 4,          // broadphase cell-change counter
    AU_STEPPED = 5,      // 1 once a world step has run (solver time step set)
    AU_ERR = 6,          // device-side error flags
    AU_EVENTS = 7,       // number of events queued this launch (capped)
    AU_COUNT = 8
};

enum DeviceError : uint32_t {
    ERR_POINT_OVERFLOW = 1u << 0,
    ERR_ROW_OVERFLOW = 1u << 1,
    ERR_PAIR_OVERFLOW = 1u << 2,
    ERR_EVENT_OVERFLOW = 1u << 3,
    ERR_NAN = 1u << 4,
    ERR_LAUNCH = 1u << 5,  // the tick kernel's grid exceeded its scratch slots; the arena was not stepped
    // not errors: contacts that the restated narrow phase does not produce yet
    WARN_EPA_SKIPPED = 1u << 8,     // box-triangle / box-sphere penetration deeper than GJK resolves
    WARN_CARCAR_SKIPPED = 1u << 9,  // overlapping car boxes (box-box detector)
};

constexpr int MAX_CARS = 8;
constexpr int NUM_PADS = 34;
constexpr int MAX_EVENTS_PER_ARENA = 64;

// ---- record word offsets
constexpr int PAD_WORDS = 4;   // cooldown (f32), then PadU fields
constexpr int CAR_WORDS = 96;  // CarF floats, then CarU words, one spare
constexpr int REC_BALL = 0;
constexpr int REC_PADS = REC_BALL + BF_COUNT + BU_COUNT;
constexpr int REC_CARS = 168;
static_assert(REC_PADS + NUM_PADS * PAD_WORDS <= REC_CARS, "record layout");
static_assert(CF_COUNT + CU_COUNT <= CAR_WORDS, "car block");
RSG_LAYOUT_FN int rec_words(int max_cars) { return REC_CARS + CAR_WORDS * max_cars; }
RSG_LAYOUT_FN int rec_ball_f(int f) { return REC_BALL + f; }
RSG_LAYOUT_FN int rec_ball_u(int f) { return REC_BALL + BF_COUNT + f; }
RSG_LAYOUT_FN int rec_pad_f(int f, int pad) { return REC_PADS + pad * PAD_WORDS + f; }
RSG_LAYOUT_FN int rec_pad_u(int f, int pad) { return REC_PADS + pad * PAD_WORDS + PF_COUNT + f; }
RSG_LAYOUT_FN int rec_car_f(int f, int slot) { return REC_CARS + slot * CAR_WORDS + f; }
RSG_LAYOUT_FN int rec_car_u(int f, int slot) { return REC_CARS + slot * CAR_WORDS + CF_COUNT + f; }

// The mutator values the tick reads (MutatorConfig, src/Sim/MutatorConfig/MutatorConfig.h:16-79),
// in the units the tick uses: gravity multiplied by UU_TO_BT as btDiscreteDynamicsWorld::setGravity
// receives it (Arena.cpp:26), the ball radius in both units.
struct MutatorsDev {
    float grav_bt[3];
    float car_world_friction, car_world_restitution;
    float ball_mass, ball_max_speed, ball_drag, ball_world_friction, ball_world_restitution;
    float jump_accel, jump_immediate_force;
    float boost_accel_ground, boost_accel_air, boost_used_per_second;
    float respawn_delay, bump_cooldown_time;
    float pad_cooldown_big, pad_cooldown_small;
    float car_spawn_boost;
    float ball_hit_scale, bump_force_scale;
    float ball_radius_uu, ball_radius_bt;
    int unlimited_flips, unlimited_double_jumps, recharge_boost;
    float recharge_per_second, recharge_delay;
    int demo_mode, team_demos;
    float goal_threshold_y;
};

// Per-car-config constants uploaded once (derived like Car::_BulletSetup, Car.cpp:195-292)
struct CarCfgDev {
    float he[3];          // box implicit half extents (without margin)
    float margin;         // box collision margin
    float off[3];         // hitbox offset
    float comp_min[3], comp_max[3];
    float inv_inertia[3];
    float breaking;       // contact breaking threshold of the compound
    float conn[4][3];     // wheel connection points (chassis space)
    float rest[2];        // suspension rest length front/back (BT)
    float radius[2];      // wheel radius front/back (BT)
    float dodge_deadzone;
    int three_wheels;
};

}  // namespace rsg
