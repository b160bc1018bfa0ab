// ref_driver.cpp -- test-only C shim over the reference RocketSim library.
//
// This file is ORACLE infrastructure: it is compiled (by oracle/Makefile) only
// where the reference source tree is present, linked against the reference's
// own sources built unmodified, and loaded only by tests/ to pin the CPU
// restatement (oracle/rs_oracle.cpp) and to write the golden fixtures under
// tests/golden/.  Nothing in the product links or loads it.
//
// It converts between the POD mirrors of include/rocketsim_gb300.h and the
// reference's CarState / BallState / BoostPadState (src/Sim/Car/Car.h:17-120,
// src/Sim/Ball/Ball.h:18-57, src/Sim/BoostPad/BoostPad.h:23-35).

#include "RocketSim.h"
#include "Sim/BallPredTracker/BallPredTracker.h"
#include "Sim/GameEventTracker/GameEventTracker.h"
#include "../libsrc/bullet3-3.24/BulletCollision/NarrowPhaseCollision/btSubSimplexConvexCast.h"
#include "../include/rocketsim_gb300.h"

#include <cstring>
#include <vector>

using namespace RocketSim;

namespace {

struct RefEvent {
    uint32_t kind;
    uint64_t tick;
    uint32_t a, b, flag;
};

struct RefArena {
    Arena* arena = nullptr;
    std::vector<RefEvent> events;
};

Vec V(const rsg_vec3& v) { return Vec(v.x, v.y, v.z); }
rsg_vec3 P(const Vec& v) { return rsg_vec3{v.x, v.y, v.z}; }

RotMat RM(const rsg_rotmat& m) { return RotMat(V(m.forward), V(m.right), V(m.up)); }
rsg_rotmat PM(const RotMat& m) { return rsg_rotmat{P(m.forward), P(m.right), P(m.up)}; }

CarControls CC(const rsg_car_controls& c) {
    CarControls r;
    r.throttle = c.throttle; r.steer = c.steer; r.pitch = c.pitch; r.yaw = c.yaw; r.roll = c.roll;
    r.jump = c.jump != 0; r.boost = c.boost != 0; r.handbrake = c.handbrake != 0;
    return r;
}
rsg_car_controls PC(const CarControls& c) {
    rsg_car_controls r{};
    r.throttle = c.throttle; r.steer = c.steer; r.pitch = c.pitch; r.yaw = c.yaw; r.roll = c.roll;
    r.jump = c.jump; r.boost = c.boost; r.handbrake = c.handbrake;
    return r;
}

void CarToPod(const CarState& s, rsg_car_state* o) {
    std::memset(o, 0, sizeof(*o));
    o->pos = P(s.pos); o->rot_mat = PM(s.rotMat); o->vel = P(s.vel); o->ang_vel = P(s.angVel);
    o->tick_count_since_update = s.tickCountSinceUpdate;
    o->is_on_ground = s.isOnGround;
    for (int i = 0; i < 4; i++) o->wheels_with_contact[i] = s.wheelsWithContact[i];
    o->has_jumped = s.hasJumped; o->has_double_jumped = s.hasDoubleJumped; o->has_flipped = s.hasFlipped;
    o->flip_rel_torque = P(s.flipRelTorque);
    o->jump_time = s.jumpTime; o->flip_time = s.flipTime;
    o->is_flipping = s.isFlipping; o->is_jumping = s.isJumping;
    o->air_time = s.airTime; o->air_time_since_jump = s.airTimeSinceJump;
    o->boost = s.boost; o->time_since_boosted = s.timeSinceBoosted;
    o->is_boosting = s.isBoosting; o->boosting_time = s.boostingTime;
    o->is_supersonic = s.isSupersonic; o->supersonic_time = s.supersonicTime;
    o->handbrake_val = s.handbrakeVal;
    o->is_auto_flipping = s.isAutoFlipping; o->auto_flip_timer = s.autoFlipTimer;
    o->auto_flip_torque_scale = s.autoFlipTorqueScale;
    o->world_contact_has_contact = s.worldContact.hasContact;
    o->world_contact_normal = P(s.worldContact.contactNormal);
    o->car_contact_other_car_id = s.carContact.otherCarID;
    o->car_contact_cooldown_timer = s.carContact.cooldownTimer;
    o->is_demoed = s.isDemoed; o->demo_respawn_timer = s.demoRespawnTimer;
    o->ball_hit_info.is_valid = s.ballHitInfo.isValid;
    o->ball_hit_info.relative_pos_on_ball = P(s.ballHitInfo.relativePosOnBall);
    o->ball_hit_info.ball_pos = P(s.ballHitInfo.ballPos);
    o->ball_hit_info.extra_hit_vel = P(s.ballHitInfo.extraHitVel);
    o->ball_hit_info.tick_count_when_hit = s.ballHitInfo.tickCountWhenHit;
    o->ball_hit_info.tick_count_when_extra_impulse_applied = s.ballHitInfo.tickCountWhenExtraImpulseApplied;
    o->last_controls = PC(s.lastControls);
}

CarState PodToCar(const rsg_car_state* o) {
    CarState s;
    s.pos = V(o->pos); s.rotMat = RM(o->rot_mat); s.vel = V(o->vel); s.angVel = V(o->ang_vel);
    s.tickCountSinceUpdate = o->tick_count_since_update;
    s.isOnGround = o->is_on_ground;
    for (int i = 0; i < 4; i++) s.wheelsWithContact[i] = o->wheels_with_contact[i];
    s.hasJumped = o->has_jumped; s.hasDoubleJumped = o->has_double_jumped; s.hasFlipped = o->has_flipped;
    s.flipRelTorque = V(o->flip_rel_torque);
    s.jumpTime = o->jump_time; s.flipTime = o->flip_time;
    s.isFlipping = o->is_flipping; s.isJumping = o->is_jumping;
    s.airTime = o->air_time; s.airTimeSinceJump = o->air_time_since_jump;
    s.boost = o->boost; s.timeSinceBoosted = o->time_since_boosted;
    s.isBoosting = o->is_boosting; s.boostingTime = o->boosting_time;
    s.isSupersonic = o->is_supersonic; s.supersonicTime = o->supersonic_time;
    s.handbrakeVal = o->handbrake_val;
    s.isAutoFlipping = o->is_auto_flipping; s.autoFlipTimer = o->auto_flip_timer;
    s.autoFlipTorqueScale = o->auto_flip_torque_scale;
    s.worldContact.hasContact = o->world_contact_has_contact;
    s.worldContact.contactNormal = V(o->world_contact_normal);
    s.carContact.otherCarID = o->car_contact_other_car_id;
    s.carContact.cooldownTimer = o->car_contact_cooldown_timer;
    s.isDemoed = o->is_demoed; s.demoRespawnTimer = o->demo_respawn_timer;
    s.ballHitInfo.isValid = o->ball_hit_info.is_valid;
    s.ballHitInfo.relativePosOnBall = V(o->ball_hit_info.relative_pos_on_ball);
    s.ballHitInfo.ballPos = V(o->ball_hit_info.ball_pos);
    s.ballHitInfo.extraHitVel = V(o->ball_hit_info.extra_hit_vel);
    s.ballHitInfo.tickCountWhenHit = o->ball_hit_info.tick_count_when_hit;
    s.ballHitInfo.tickCountWhenExtraImpulseApplied = o->ball_hit_info.tick_count_when_extra_impulse_applied;
    s.lastControls = CC(o->last_controls);
    return s;
}

const CarConfig* PRESETS[6] = {&CAR_CONFIG_OCTANE, &CAR_CONFIG_DOMINUS, &CAR_CONFIG_PLANK,
                               &CAR_CONFIG_BREAKOUT, &CAR_CONFIG_HYBRID, &CAR_CONFIG_MERC};

void OnGoal(Arena* arena, Team team, void* user) {
    RefArena* ra = (RefArena*)user;
    ra->events.push_back({RSG_EVENT_GOAL, arena->tickCount, (uint32_t)team, 0, 0});
}

void OnBump(Arena* arena, Car* bumper, Car* victim, bool isDemo, void* user) {
    RefArena* ra = (RefArena*)user;
    ra->events.push_back({RSG_EVENT_BUMP, arena->tickCount, bumper->id, victim->id, (uint32_t)isDemo});
}

Car* FindCar(RefArena* ra, uint32_t id) {
    for (Car* c : ra->arena->GetCars())
        if (c->id == id) return c;
    return nullptr;
}

}  // namespace

extern "C" {

int rsref_init(const uint8_t* cmf, uint64_t len) {
    std::map<GameMode, std::vector<FileData>> m;
    FileData fd(cmf, cmf + len);
    m[GameMode::SOCCAR].push_back(fd);
    m[GameMode::HEATSEEKER].push_back(fd);  // heatseeker plays in the soccar arena
    try {
        RocketSim::InitFromMem(m, true);
    } catch (...) {
        return -1;
    }
    return 0;
}

void* rsref_arena_create(int game_mode, float tick_rate) {
    RefArena* ra = new RefArena();
    try {
        ra->arena = Arena::Create((GameMode)game_mode, ArenaConfig(), tick_rate);
    } catch (...) {
        delete ra;
        return nullptr;
    }
    ra->arena->SetCarBumpCallback(OnBump, ra);
    if ((GameMode)game_mode != GameMode::THE_VOID) ra->arena->SetGoalScoreCallback(OnGoal, ra);
    return ra;
}

// Arena::Create with an ArenaConfig from its POD mirror (ArenaConfig.h:19-50)
void* rsref_arena_create_ex(int game_mode, float tick_rate, const rsg_arena_config* c) {
    ArenaConfig cfg;
    cfg.memWeightMode = (ArenaMemWeightMode)c->mem_weight_mode;
    cfg.minPos = V(c->min_pos);
    cfg.maxPos = V(c->max_pos);
    cfg.maxAABBLen = c->max_aabb_len;
    cfg.noBallRot = c->no_ball_rot != 0;
    cfg.useCustomBroadphase = c->use_custom_broadphase != 0;
    cfg.maxObjects = c->max_objects;
    cfg.useCustomBoostPads = c->use_custom_boost_pads != 0;
    for (uint32_t i = 0; i < c->num_custom_boost_pads; i++) {
        BoostPadConfig pc;
        pc.pos = V(c->custom_boost_pads[i].pos);
        pc.isBig = c->custom_boost_pads[i].is_big != 0;
        cfg.customBoostPads.push_back(pc);
    }
    RefArena* ra = new RefArena();
    try {
        ra->arena = Arena::Create((GameMode)game_mode, cfg, tick_rate);
    } catch (...) {
        delete ra;
        return nullptr;
    }
    ra->arena->SetCarBumpCallback(OnBump, ra);
    if ((GameMode)game_mode != GameMode::THE_VOID) ra->arena->SetGoalScoreCallback(OnGoal, ra);
    return ra;
}

void rsref_arena_destroy(void* h) {
    RefArena* ra = (RefArena*)h;
    delete ra->arena;
    delete ra;
}

int rsref_preset(int preset, rsg_car_config* out) {
    if (preset < 0 || preset > 5) return -1;
    const CarConfig& c = *PRESETS[preset];
    std::memset(out, 0, sizeof(*out));
    out->hitbox_size = P(c.hitboxSize);
    out->hitbox_pos_offset = P(c.hitboxPosOffset);
    out->front_wheels.wheel_radius = c.frontWheels.wheelRadius;
    out->front_wheels.suspension_rest_length = c.frontWheels.suspensionRestLength;
    out->front_wheels.connection_point_offset = P(c.frontWheels.connectionPointOffset);
    out->back_wheels.wheel_radius = c.backWheels.wheelRadius;
    out->back_wheels.suspension_rest_length = c.backWheels.suspensionRestLength;
    out->back_wheels.connection_point_offset = P(c.backWheels.connectionPointOffset);
    out->three_wheels = c.threeWheels;
    out->dodge_deadzone = c.dodgeDeadzone;
    return 0;
}

uint32_t rsref_add_car(void* h, int team, int preset) {
    RefArena* ra = (RefArena*)h;
    Car* c = ra->arena->AddCar((Team)team, *PRESETS[preset]);
    return c->id;
}

int rsref_car_order(void* h, uint32_t* out, uint32_t cap) {
    RefArena* ra = (RefArena*)h;
    uint32_t n = 0;
    for (Car* c : ra->arena->GetCars()) {
        if (n < cap) out[n] = c->id;
        n++;
    }
    return (int)n;
}

int rsref_set_controls(void* h, uint32_t id, const rsg_car_controls* c) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    car->controls = CC(*c);
    return 0;
}

int rsref_get_car(void* h, uint32_t id, rsg_car_state* out) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    CarToPod(car->GetState(), out);
    return 0;
}

int rsref_set_car(void* h, uint32_t id, const rsg_car_state* s) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    car->SetState(PodToCar(s));
    return 0;
}

int rsref_get_ball(void* h, rsg_ball_state* out) {
    RefArena* ra = (RefArena*)h;
    BallState s = ra->arena->ball->GetState();
    std::memset(out, 0, sizeof(*out));
    out->pos = P(s.pos); out->rot_mat = PM(s.rotMat); out->vel = P(s.vel); out->ang_vel = P(s.angVel);
    out->tick_count_since_update = s.tickCountSinceUpdate;
    return 0;
}

int rsref_set_ball(void* h, const rsg_ball_state* in) {
    RefArena* ra = (RefArena*)h;
    BallState s;
    s.pos = V(in->pos); s.rotMat = RM(in->rot_mat); s.vel = V(in->vel); s.angVel = V(in->ang_vel);
    ra->arena->ball->SetState(s);
    return 0;
}

// BallPredTracker over an arena of this driver (the tracker makes its own ball-only arena).
static BallState PodToBall(const rsg_ball_state* in) {
    BallState s;
    s.pos = V(in->pos); s.rotMat = RM(in->rot_mat); s.vel = V(in->vel); s.angVel = V(in->ang_vel);
    s.tickCountSinceUpdate = in->tick_count_since_update;
    return s;
}
static void BallToPod(const BallState& s, rsg_ball_state* out) {
    std::memset(out, 0, sizeof(*out));
    out->pos = P(s.pos); out->rot_mat = PM(s.rotMat); out->vel = P(s.vel); out->ang_vel = P(s.angVel);
    out->tick_count_since_update = s.tickCountSinceUpdate;
}
void* rsref_ballpred_create(void* h, uint32_t num_pred_ticks) {
    return new BallPredTracker(((RefArena*)h)->arena, num_pred_ticks);
}
void rsref_ballpred_destroy(void* t) { delete (BallPredTracker*)t; }
void rsref_ballpred_update_from_arena(void* t, void* h) { ((BallPredTracker*)t)->UpdatePredFromArena(((RefArena*)h)->arena); }
void rsref_ballpred_update_manual(void* t, const rsg_ball_state* cur, int ticks) {
    ((BallPredTracker*)t)->UpdatePredManual(PodToBall(cur), ticks);
}
void rsref_ballpred_force_update_all(void* t, const rsg_ball_state* initial) {
    ((BallPredTracker*)t)->ForceUpdateAllPred(PodToBall(initial));
}
// predData (out[cap]); returns its size
int rsref_ballpred_get(void* t, rsg_ball_state* out, int cap) {
    auto& d = ((BallPredTracker*)t)->predData;
    for (int i = 0; i < (int)d.size() && i < cap; i++) BallToPod(d[i], out + i);
    return (int)d.size();
}
void rsref_ballpred_state_for_time(void* t, float pred_time, rsg_ball_state* out) {
    BallToPod(((BallPredTracker*)t)->GetBallStateForTime(pred_time), out);
}
int rsref_ballpred_last_update_tick(void* t) { return ((BallPredTracker*)t)->lastUpdateTickCount; }

void rsref_reset_to_random_kickoff(void* h, int seed) { ((RefArena*)h)->arena->ResetToRandomKickoff(seed); }
// Arena::IsBallProbablyGoingIn; *team = the goal's team, or -1
int rsref_is_ball_probably_going_in(void* h, float max_time, float extra_margin, int* team) {
    Team t = Team::BLUE;
    bool in = ((RefArena*)h)->arena->IsBallProbablyGoingIn(max_time, extra_margin, &t);
    *team = in ? (int)t : -1;
    return in ? 1 : 0;
}

// GameEventTracker with callbacks that record the event of the last Update (kind 1 shot, 2 goal,
// 3 save; ids of the cars, 0 for none).
struct RefEventTracker {
    GameEventTracker t;
    int ev[3] = {0, 0, 0};
};
void* rsref_gevt_create(const float* cfg7, int auto_detect) {
    RefEventTracker* r = new RefEventTracker();
    GameEventTrackerConfig& c = r->t.config;
    c.shotMinSpeed = cfg7[0]; c.shotTouchMinDelay = cfg7[1]; c.predScoreExtraMargin = cfg7[2];
    c.shotEventCooldown = cfg7[3]; c.shotMinScoreTime = cfg7[4]; c.goalMaxTouchTime = cfg7[5]; c.passMaxTouchTime = cfg7[6];
    r->t.autoStateSetDetection = auto_detect != 0;
    auto id = [](Car* c) { return c ? (int)c->id : 0; };
    r->t.SetShotCallback([id](Arena*, Car* s, Car* p, void* u) { int* e = (int*)u; e[0] = 1; e[1] = id(s); e[2] = id(p); }, r->ev);
    r->t.SetGoalCallback([id](Arena*, Car* s, Car* p, void* u) { int* e = (int*)u; e[0] = 2; e[1] = id(s); e[2] = id(p); }, r->ev);
    r->t.SetSaveCallback([id](Arena*, Car* s, void* u) { int* e = (int*)u; e[0] = 3; e[1] = id(s); e[2] = 0; }, r->ev);
    return r;
}
void rsref_gevt_update(void* t, void* h, int* out3) {
    RefEventTracker* r = (RefEventTracker*)t;
    r->ev[0] = r->ev[1] = r->ev[2] = 0;
    r->t.Update(((RefArena*)h)->arena);
    out3[0] = r->ev[0]; out3[1] = r->ev[1]; out3[2] = r->ev[2];
}
void rsref_gevt_reset(void* t) { ((RefEventTracker*)t)->t.ResetPersistentInfo(); }
void rsref_gevt_destroy(void* t) { delete (RefEventTracker*)t; }

int rsref_num_pads(void* h) { return (int)((RefArena*)h)->arena->GetBoostPads().size(); }

int rsref_get_pad(void* h, int i, rsg_pad_state* out) {
    RefArena* ra = (RefArena*)h;
    auto& pads = ra->arena->GetBoostPads();
    if (i < 0 || i >= (int)pads.size()) return -1;
    BoostPadState s = pads[i]->GetState();
    std::memset(out, 0, sizeof(*out));
    out->is_active = s.isActive;
    out->cooldown = s.cooldown;
    out->cur_locked_car_id = s.curLockedCar ? s.curLockedCar->id : 0;
    out->prev_locked_car_id = s.prevLockedCarID;
    return 0;
}

int rsref_set_pad(void* h, int i, const rsg_pad_state* in) {
    RefArena* ra = (RefArena*)h;
    auto& pads = ra->arena->GetBoostPads();
    if (i < 0 || i >= (int)pads.size()) return -1;
    BoostPadState s;
    s.isActive = in->is_active;
    s.cooldown = in->cooldown;
    s.curLockedCar = nullptr;
    s.prevLockedCarID = in->prev_locked_car_id;
    pads[i]->SetState(s);
    return 0;
}

int rsref_pad_config(void* h, int i, rsg_vec3* pos, int* is_big) {
    RefArena* ra = (RefArena*)h;
    auto& pads = ra->arena->GetBoostPads();
    if (i < 0 || i >= (int)pads.size()) return -1;
    *pos = P(pads[i]->config.pos);
    *is_big = pads[i]->config.isBig;
    return 0;
}

uint64_t rsref_get_tick(void* h) { return ((RefArena*)h)->arena->tickCount; }
void rsref_set_tick(void* h, uint64_t t) { ((RefArena*)h)->arena->tickCount = t; }

int rsref_step(void* h, int ticks) {
    RefArena* ra = (RefArena*)h;
    try {
        ra->arena->Step(ticks);
    } catch (...) {
        return -1;
    }
    return 0;
}

// Steps `ticks` ticks, setting the controls of car k (in AddCar order, ids 1..n) from
// controls[t * ncars + k] before tick t.  Used to time the reference without a
// per-tick round trip through the caller's language.
int rsref_run(void* h, const rsg_car_controls* controls, int ncars, int ticks) {
    RefArena* ra = (RefArena*)h;
    std::vector<Car*> cars;
    for (int k = 0; k < ncars; k++) {
        Car* c = FindCar(ra, (uint32_t)(k + 1));
        if (!c) return -1;
        cars.push_back(c);
    }
    try {
        for (int t = 0; t < ticks; t++) {
            for (int k = 0; k < ncars; k++) cars[k]->controls = CC(controls[(size_t)t * ncars + k]);
            ra->arena->Step(1);
        }
    } catch (...) {
        return -1;
    }
    return 0;
}

int rsref_is_scored(void* h) { return ((RefArena*)h)->arena->IsBallScored() ? 1 : 0; }

// Events recorded since the last call: each event is 5 uint64 words
// (kind, tick, a, b, flag).  Returns the number of events copied.
int rsref_pop_events(void* h, uint64_t* out, int cap) {
    RefArena* ra = (RefArena*)h;
    int n = 0;
    for (auto& e : ra->events) {
        if (n >= cap) break;
        out[n * 5 + 0] = e.kind;
        out[n * 5 + 1] = e.tick;
        out[n * 5 + 2] = e.a;
        out[n * 5 + 3] = e.b;
        out[n * 5 + 4] = e.flag;
        n++;
    }
    ra->events.clear();
    return n;
}

// Wheel internals of btVehicleRL (src/Sim/btVehicleRL/btVehicleRL.h:9-27) that
// persist across ticks but are not part of CarState: steer angle and extra
// pushback per wheel.  Used by tests to check the restatement's hidden state.
int rsref_get_wheel_internals(void* h, uint32_t id, float* out8) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    for (int i = 0; i < 4; i++) {
        out8[i] = car->_bulletVehicle.m_wheelInfo[i].m_steerAngle;
        out8[4 + i] = car->_bulletVehicle.m_wheelInfo[i].m_extraPushback;
    }
    return 0;
}

// Arena::Serialize into `out` (DataStreamOut's bytes, no version word); *len receives the size.
int rsref_serialize(void* h, uint8_t* out, uint64_t cap, uint64_t* len) {
    DataStreamOut o;
    ((RefArena*)h)->arena->Serialize(o);
    *len = o.data.size();
    if (out && cap >= o.data.size()) std::memcpy(out, o.data.data(), o.data.size());
    return 0;
}

// Arena::DeserializeNew from bytes; a new arena handle (NULL on failure).
void* rsref_deserialize_new(const uint8_t* data, uint64_t len) {
    DataStreamIn in;
    in.data.assign(data, data + len);
    RefArena* ra = new RefArena();
    try {
        ra->arena = Arena::DeserializeNew(in);
    } catch (...) {
        delete ra;
        return nullptr;
    }
    ra->arena->SetCarBumpCallback(OnBump, ra);
    if (ra->arena->gameMode != GameMode::THE_VOID) ra->arena->SetGoalScoreCallback(OnGoal, ra);
    return ra;
}

// Arena::Clone (without the callbacks, which are set to this driver's own); a new arena handle.
void* rsref_clone(void* h) {
    RefArena* ra = new RefArena();
    ra->arena = ((RefArena*)h)->arena->Clone(false);
    ra->arena->SetCarBumpCallback(OnBump, ra);
    if (ra->arena->gameMode != GameMode::THE_VOID) ra->arena->SetGoalScoreCallback(OnGoal, ra);
    return ra;
}

// Arena::SetMutatorConfig / MutatorConfig(GameMode) through the POD mirror
// (src/Sim/MutatorConfig/MutatorConfig.h:16-79, field for field).
int rsref_set_mutator_config(void* h, const rsg_mutator_config* c) {
    RefArena* ra = (RefArena*)h;
    MutatorConfig m = ra->arena->GetMutatorConfig();
    m.gravity = V(c->gravity);
    m.carMass = c->car_mass;
    m.carWorldFriction = c->car_world_friction;
    m.carWorldRestitution = c->car_world_restitution;
    m.ballMass = c->ball_mass;
    m.ballMaxSpeed = c->ball_max_speed;
    m.ballDrag = c->ball_drag;
    m.ballWorldFriction = c->ball_world_friction;
    m.ballWorldRestitution = c->ball_world_restitution;
    m.jumpAccel = c->jump_accel;
    m.jumpImmediateForce = c->jump_immediate_force;
    m.boostAccelGround = c->boost_accel_ground;
    m.boostAccelAir = c->boost_accel_air;
    m.boostUsedPerSecond = c->boost_used_per_second;
    m.respawnDelay = c->respawn_delay;
    m.bumpCooldownTime = c->bump_cooldown_time;
    m.boostPadCooldown_Big = c->boost_pad_cooldown_big;
    m.boostPadCooldown_Small = c->boost_pad_cooldown_small;
    m.carSpawnBoostAmount = c->car_spawn_boost_amount;
    m.ballHitExtraForceScale = c->ball_hit_extra_force_scale;
    m.bumpForceScale = c->bump_force_scale;
    m.ballRadius = c->ball_radius;
    m.unlimitedFlips = c->unlimited_flips != 0;
    m.unlimitedDoubleJumps = c->unlimited_double_jumps != 0;
    m.rechargeBoostEnabled = c->recharge_boost_enabled != 0;
    m.rechargeBoostPerSecond = c->recharge_boost_per_second;
    m.rechargeBoostDelay = c->recharge_boost_delay;
    m.demoMode = (DemoMode)c->demo_mode;
    m.enableTeamDemos = c->enable_team_demos != 0;
    m.goalBaseThresholdY = c->goal_base_threshold_y;
    ra->arena->SetMutatorConfig(m);
    return 0;
}

int rsref_default_mutator_config(int game_mode, rsg_mutator_config* o) {
    MutatorConfig m((GameMode)game_mode);
    std::memset(o, 0, sizeof(*o));
    o->gravity = rsg_vec3{m.gravity.x, m.gravity.y, m.gravity.z};
    o->car_mass = m.carMass;
    o->car_world_friction = m.carWorldFriction;
    o->car_world_restitution = m.carWorldRestitution;
    o->ball_mass = m.ballMass;
    o->ball_max_speed = m.ballMaxSpeed;
    o->ball_drag = m.ballDrag;
    o->ball_world_friction = m.ballWorldFriction;
    o->ball_world_restitution = m.ballWorldRestitution;
    o->jump_accel = m.jumpAccel;
    o->jump_immediate_force = m.jumpImmediateForce;
    o->boost_accel_ground = m.boostAccelGround;
    o->boost_accel_air = m.boostAccelAir;
    o->boost_used_per_second = m.boostUsedPerSecond;
    o->respawn_delay = m.respawnDelay;
    o->bump_cooldown_time = m.bumpCooldownTime;
    o->boost_pad_cooldown_big = m.boostPadCooldown_Big;
    o->boost_pad_cooldown_small = m.boostPadCooldown_Small;
    o->car_spawn_boost_amount = m.carSpawnBoostAmount;
    o->ball_hit_extra_force_scale = m.ballHitExtraForceScale;
    o->bump_force_scale = m.bumpForceScale;
    o->ball_radius = m.ballRadius;
    o->unlimited_flips = m.unlimitedFlips;
    o->unlimited_double_jumps = m.unlimitedDoubleJumps;
    o->recharge_boost_enabled = m.rechargeBoostEnabled;
    o->recharge_boost_per_second = m.rechargeBoostPerSecond;
    o->recharge_boost_delay = m.rechargeBoostDelay;
    o->demo_mode = (uint8_t)m.demoMode;
    o->enable_team_demos = m.enableTeamDemos;
    o->goal_base_threshold_y = m.goalBaseThresholdY;
    return 0;
}

// The vehicle state the next tick starts from that CarState leaves out (btVehicleRL.h:9-27,
// btWheelInfo.h:73-101): front steer angle, engine force, brake, then per wheel the lateral and
// longitudinal friction factors and the extra push-back (15 floats).
int rsref_get_vehicle_state(void* h, uint32_t id, float* out15) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    auto& wi = car->_bulletVehicle.m_wheelInfo;
    out15[0] = wi[0].m_steerAngle;
    out15[1] = wi[0].m_engineForce;
    out15[2] = wi[0].m_brake;
    for (int i = 0; i < 4; i++) {
        out15[3 + i] = wi[i].m_latFriction;
        out15[7 + i] = wi[i].m_longFriction;
        out15[11 + i] = wi[i].m_extraPushback;
    }
    return 0;
}

}  // extern "C"

extern "C" {
// Per-wheel raycast/friction internals for debugging the restatement:
// 16 floats per wheel: contact point(3) normal(3) susp_len rel_vel clipped_inv
// impulse(3) lat long hard_point.z ground(0 none,1 static,2 dynamic)
int rsref_wheel_debug(void* h, uint32_t id, float* out) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    for (int i = 0; i < 4; i++) {
        auto& w = car->_bulletVehicle.m_wheelInfo[i];
        float* o = out + i * 16;
        o[0] = w.m_raycastInfo.m_contactPointWS.x(); o[1] = w.m_raycastInfo.m_contactPointWS.y(); o[2] = w.m_raycastInfo.m_contactPointWS.z();
        o[3] = w.m_raycastInfo.m_contactNormalWS.x(); o[4] = w.m_raycastInfo.m_contactNormalWS.y(); o[5] = w.m_raycastInfo.m_contactNormalWS.z();
        o[6] = w.m_raycastInfo.m_suspensionLength; o[7] = w.m_suspensionRelativeVelocity; o[8] = w.m_clippedInvContactDotSuspension;
        o[9] = w.m_impulse.x(); o[10] = w.m_impulse.y(); o[11] = w.m_impulse.z();
        o[12] = w.m_latFriction; o[13] = w.m_longFriction; o[14] = w.m_raycastInfo.m_hardPointWS.z();
        const btCollisionObject* g = (const btCollisionObject*)w.m_raycastInfo.m_groundObject;
        o[15] = g ? (g->isStaticObject() ? 1.f : 2.f) : 0.f;
    }
    return 0;
}
}

extern "C" {
// Rigid-body internals of a car: inv inertia local(3), inv mass, inv inertia world(9)
int rsref_body_debug(void* h, uint32_t id, float* out) {
    Car* car = FindCar((RefArena*)h, id);
    if (!car) return -1;
    btVector3 il = car->_rigidBody.getInvInertiaDiagLocal();
    out[0] = il.x(); out[1] = il.y(); out[2] = il.z();
    out[3] = car->_rigidBody.getInvMass();
    const btMatrix3x3& m = car->_rigidBody.getInvInertiaTensorWorld();
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) out[4 + i * 3 + j] = m[i][j];
    btVector3 he = car->_childHitboxShape.getHalfExtentsWithoutMargin();
    out[13] = he.x(); out[14] = he.y(); out[15] = he.z(); out[16] = car->_childHitboxShape.getMargin();
    return 0;
}
}

extern "C" {
// btCollisionWorld::rayTest from `in6` (from, to; Bullet units) with a ClosestRayResultCallback that
// ignores car `ignore_id` (0: none), as the vehicle raycaster runs it (test aid): writes hit (0/1),
// fraction, normal (3), object kind (0 none, 1 static, 2 ball, 3 car) and car id.
int rsref_debug_ray(void* h, const float* in6, uint32_t ignore_id, float* out7) {
    RefArena* ra = (RefArena*)h;
    btVector3 from(in6[0], in6[1], in6[2]), to(in6[3], in6[4], in6[5]);
    Car* ign = ignore_id ? FindCar(ra, ignore_id) : nullptr;
    btCollisionWorld::ClosestRayResultCallback cb(from, to, ign ? (const btCollisionObject*)&ign->_rigidBody : nullptr);
    ra->arena->_bulletWorld.rayTest(from, to, cb);
    out7[0] = cb.hasHit() ? 1.f : 0.f;
    out7[1] = cb.m_closestHitFraction;
    out7[2] = cb.m_hitNormalWorld.x(); out7[3] = cb.m_hitNormalWorld.y(); out7[4] = cb.m_hitNormalWorld.z();
    out7[5] = 0; out7[6] = 0;
    if (cb.hasHit()) {
        const btCollisionObject* o = cb.m_collisionObject;
        out7[5] = o->isStaticObject() ? 1.f : 0.f;
        if (o == &ra->arena->ball->_rigidBody) out7[5] = 2.f;
        for (Car* c : ra->arena->GetCars())
            if (o == &c->_rigidBody) { out7[5] = 3.f; out7[6] = (float)c->id; }
    }
    return 0;
}
}

extern "C" {
// btSubsimplexConvexCast of a point from in6[0:3] to in6[3:6] against the box child of car `car_id`
// (test aid): writes the fraction and hit (2 floats), then the same loop restated here with the
// reference's own solver and shapes, traced per iteration (lambda, v, dist2, vertices: 6 floats).
int rsref_debug_subsimplex(void* h, const float* in6, uint32_t car_id, float* out, int cap) {
    RefArena* ra = (RefArena*)h;
    Car* car = FindCar(ra, car_id);
    if (!car) return -1;
    btTransform fromT, toT;
    fromT.setIdentity(); toT.setIdentity();
    fromT.setOrigin(btVector3(in6[0], in6[1], in6[2]));
    toT.setOrigin(btVector3(in6[3], in6[4], in6[5]));
    const btCompoundShape* comp = (const btCompoundShape*)car->_rigidBody.getCollisionShape();
    const btConvexShape* box = (const btConvexShape*)comp->getChildShape(0);
    btTransform childW = car->_rigidBody.getWorldTransform() * comp->getChildTransform(0);
    btSphereShape pointShape(btScalar(0.0));
    pointShape.setMargin(0.f);
    {
        btVoronoiSimplexSolver ss;
        btSubsimplexConvexCast cc(&pointShape, box, &ss);
        btConvexCast::CastResult res;
        res.m_fraction = 1.f;
        bool ok = cc.calcTimeOfImpact(fromT, toT, childW, childW, res);
        out[0] = res.m_fraction; out[1] = ok;
    }
    btVoronoiSimplexSolver sx;
    sx.reset();
    btVector3 r = toT.getOrigin() - fromT.getOrigin();
    btScalar lambda = 0;
    btTransform ia = fromT;
    btVector3 sa = fromT(pointShape.localGetSupportingVertex(-r * fromT.getBasis()));
    btVector3 sb = childW(box->localGetSupportingVertex(r * childW.getBasis()));
    btVector3 v = sa - sb, w;
    btScalar dist2 = v.length2();
    int maxIter = 32, n = 0;
    while ((dist2 > btScalar(0.0001)) && maxIter--) {
        sa = ia(pointShape.localGetSupportingVertex(-v * ia.getBasis()));
        sb = childW(box->localGetSupportingVertex(v * childW.getBasis()));
        w = sa - sb;
        btScalar vdw = v.dot(w);
        if (lambda > 1) break;
        if (vdw > 0) {
            btScalar vdr = v.dot(r);
            if (vdr >= -(SIMD_EPSILON * SIMD_EPSILON)) break;
            lambda = lambda - vdw / vdr;
            ia.getOrigin().setInterpolate3(fromT.getOrigin(), toT.getOrigin(), lambda);
            w = sa - sb;
        }
        if (!sx.inSimplex(w)) sx.addVertex(w, sa, sb);
        if (sx.closest(v)) dist2 = v.length2(); else dist2 = 0;
        if (n < cap) {
            float* o = out + 2 + 6 * n;
            o[0] = lambda; o[1] = v.x(); o[2] = v.y(); o[3] = v.z(); o[4] = dist2; o[5] = sx.numVertices();
        }
        n++;
    }
    return n;
}
}

extern "C" {
// BallState::hsInfo of the arena's ball: yTargetDir, curTargetSpeed, timeSinceHit (test aid).
int rsref_get_ball_hs(void* h, float* out3) {
    BallState st = ((RefArena*)h)->arena->ball->GetState();
    out3[0] = st.hsInfo.yTargetDir;
    out3[1] = st.hsInfo.curTargetSpeed;
    out3[2] = st.hsInfo.timeSinceHit;
    return 0;
}
}

extern "C" {
// Sets BallState::hsInfo through Ball::SetState with the ball's current state (test aid).
int rsref_set_ball_hs(void* h, const float* in3) {
    Ball* ball = ((RefArena*)h)->arena->ball;
    BallState st = ball->GetState();
    st.hsInfo.yTargetDir = in3[0];
    st.hsInfo.curTargetSpeed = in3[1];
    st.hsInfo.timeSinceHit = in3[2];
    ball->SetState(st);
    return 0;
}
}
