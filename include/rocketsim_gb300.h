/*
 * rocketsim_gb300.h -- C ABI of the GB300-native RocketSim arena tick.
 *
 * Every entry point replaces one call of RocketSim's C++ Arena/Car/Ball API
 * (ZealanL/RocketSim v2.2); the reference interface each one stands in for is
 * cited beside it as <file>:<line> relative to the RocketSim source tree.
 *
 * Rules of the ABI:
 *  - plain C types only (no torch, no C++ classes); all structs are POD with
 *    explicit padding so that ctypes / cgo / JNI mirrors can be written by hand;
 *  - every function returns int status (RSG_OK == 0) or a pointer (NULL on
 *    error); the message of the last error on the calling thread is returned
 *    by rsg_get_last_error().  Nothing throws across this boundary
 *    (the reference throws std::runtime_error, src/Framework.h:67-72);
 *  - state crosses the boundary in Unreal units (uu) exactly like
 *    Car::GetState / Car::SetState (src/Sim/Car/Car.cpp:10-36) and
 *    Ball::GetState / Ball::SetState (src/Sim/Ball/Ball.cpp:27-51); inside the
 *    library it is kept in Bullet units (uu / 50) as the reference does;
 *  - a batch owns many independent arenas that live in device memory as
 *    structure-of-arrays; calls on one batch must be externally serialised
 *    (the reference arena is not thread-safe either, src/Sim/Arena/Arena.h).
 */
#ifndef ROCKETSIM_GB300_H
#define ROCKETSIM_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSG_OK 0
#define RSG_ERR_ARG (-1)        /* bad argument (index, size, null pointer) */
#define RSG_ERR_STATE (-2)      /* call not valid in the current state */
#define RSG_ERR_CUDA (-3)       /* a CUDA runtime call failed */
#define RSG_ERR_MESH (-4)       /* collision mesh file rejected */
#define RSG_ERR_DEVICE (-5)     /* a kernel reported a device-side error flag */

/* Game modes: src/Sim/GameMode.h:6-17. Only SOCCAR and THE_VOID are simulated. */
#define RSG_GAMEMODE_SOCCAR 0
#define RSG_GAMEMODE_HEATSEEKER 2
#define RSG_GAMEMODE_THE_VOID 5

/* Teams: src/Sim/Car/Car.h:130-133 */
#define RSG_TEAM_BLUE 0
#define RSG_TEAM_ORANGE 1

/* Car hitbox presets: src/Sim/Car/CarConfig/CarConfig.cpp:94-100 */
#define RSG_CAR_OCTANE 0
#define RSG_CAR_DOMINUS 1
#define RSG_CAR_PLANK 2
#define RSG_CAR_BREAKOUT 3
#define RSG_CAR_HYBRID 4
#define RSG_CAR_MERC 5

#define RSG_MAX_CARS_PER_ARENA 8
#define RSG_NUM_BOOST_PADS 34

typedef struct rsg_vec3 {
    float x, y, z;
} rsg_vec3;

/* Column vectors forward/right/up, src/Math/MathTypes/MathTypes.h:169-176 */
typedef struct rsg_rotmat {
    rsg_vec3 forward, right, up;
} rsg_rotmat;

/* CarControls, src/Sim/CarControls.h:7-33 (bools stored as uint8_t) */
typedef struct rsg_car_controls {
    float throttle, steer, pitch, yaw, roll;
    uint8_t jump, boost, handbrake, _pad0;
} rsg_car_controls;

/* BallHitInfo, src/Sim/BallHitInfo/BallHitInfo.h:9-26 */
typedef struct rsg_ball_hit_info {
    uint8_t is_valid;
    uint8_t _pad0[3];
    rsg_vec3 relative_pos_on_ball;
    rsg_vec3 ball_pos;
    rsg_vec3 extra_hit_vel;
    uint64_t tick_count_when_hit;
    uint64_t tick_count_when_extra_impulse_applied;
} rsg_ball_hit_info;

/* CarState, src/Sim/Car/Car.h:17-120, field for field */
typedef struct rsg_car_state {
    rsg_vec3 pos;
    rsg_rotmat rot_mat;
    rsg_vec3 vel;
    rsg_vec3 ang_vel;
    uint64_t tick_count_since_update;
    uint8_t is_on_ground;
    uint8_t wheels_with_contact[4];
    uint8_t has_jumped;
    uint8_t has_double_jumped;
    uint8_t has_flipped;
    rsg_vec3 flip_rel_torque;
    float jump_time;
    float flip_time;
    uint8_t is_flipping;
    uint8_t is_jumping;
    uint8_t _pad0[2];
    float air_time;
    float air_time_since_jump;
    float boost;
    float time_since_boosted;
    uint8_t is_boosting;
    uint8_t _pad1[3];
    float boosting_time;
    uint8_t is_supersonic;
    uint8_t _pad2[3];
    float supersonic_time;
    float handbrake_val;
    uint8_t is_auto_flipping;
    uint8_t _pad3[3];
    float auto_flip_timer;
    float auto_flip_torque_scale;
    uint8_t world_contact_has_contact;
    uint8_t _pad4[3];
    rsg_vec3 world_contact_normal;
    uint32_t car_contact_other_car_id;
    float car_contact_cooldown_timer;
    uint8_t is_demoed;
    uint8_t _pad5[3];
    float demo_respawn_timer;
    rsg_ball_hit_info ball_hit_info;
    rsg_car_controls last_controls;
} rsg_car_state;

/* BallState, src/Sim/Ball/Ball.h:18-57 (soccar part) */
typedef struct rsg_ball_state {
    rsg_vec3 pos;
    rsg_rotmat rot_mat;
    rsg_vec3 vel;
    rsg_vec3 ang_vel;
    uint64_t tick_count_since_update;
} rsg_ball_state;

/* BallState::HeatseekerInfo, src/Sim/Ball/Ball.h:24-32 (heatseeker's seeking ball) */
typedef struct rsg_heatseeker_info {
    float y_target_dir;      /* the net the ball seeks: 1 orange (+y), -1 blue, 0 none */
    float cur_target_speed;  /* uu/s */
    float time_since_hit;    /* s */
} rsg_heatseeker_info;

/* BoostPadState, src/Sim/BoostPad/BoostPad.h:23-35 */
typedef struct rsg_pad_state {
    uint8_t is_active;
    uint8_t _pad0[3];
    float cooldown;
    uint32_t cur_locked_car_id;
    uint32_t prev_locked_car_id;
} rsg_pad_state;

/* WheelPairConfig / CarConfig, src/Sim/Car/CarConfig/CarConfig.h:5-40 */
typedef struct rsg_wheel_pair_config {
    float wheel_radius;
    float suspension_rest_length;
    rsg_vec3 connection_point_offset;
} rsg_wheel_pair_config;

typedef struct rsg_car_config {
    rsg_vec3 hitbox_size;
    rsg_vec3 hitbox_pos_offset;
    rsg_wheel_pair_config front_wheels;
    rsg_wheel_pair_config back_wheels;
    uint8_t three_wheels;
    uint8_t _pad0[3];
    float dodge_deadzone;
} rsg_car_config;

/* BoostPadConfig (src/Sim/BoostPad/BoostPad.h:14-18) */
typedef struct rsg_boost_pad_config {
    rsg_vec3 pos;
    uint8_t is_big;
    uint8_t _pad0[3];
} rsg_boost_pad_config;

/* ArenaConfig (src/Sim/Arena/ArenaConfig/ArenaConfig.h:19-50), field for field.
 * custom_boost_pads is a host array of num_custom_boost_pads entries, read at
 * batch creation.  The batch holds up to 34 pads per arena, keeps the broadphase
 * of the default min_pos / max_pos / max_aabb_len / use_custom_broadphase
 * (other values return RSG_ERR_ARG), and sizes its memory by the batch
 * (mem_weight_mode and max_objects are accepted and have no effect). */
typedef struct rsg_arena_config {
    uint8_t mem_weight_mode;
    uint8_t no_ball_rot;
    uint8_t use_custom_broadphase;
    uint8_t use_custom_boost_pads;
    rsg_vec3 min_pos;
    rsg_vec3 max_pos;
    float max_aabb_len;
    int32_t max_objects;
    uint32_t num_custom_boost_pads;
    const rsg_boost_pad_config* custom_boost_pads;
} rsg_arena_config;

/* MutatorConfig (src/Sim/MutatorConfig/MutatorConfig.h:16-79), field for field,
 * uu units like the reference.  demo_mode: 0 normal, 1 on contact, 2 disabled. */
typedef struct rsg_mutator_config {
    rsg_vec3 gravity;
    float car_mass;
    float car_world_friction;
    float car_world_restitution;
    float ball_mass;
    float ball_max_speed;
    float ball_drag;
    float ball_world_friction;
    float ball_world_restitution;
    float jump_accel;
    float jump_immediate_force;
    float boost_accel_ground;
    float boost_accel_air;
    float boost_used_per_second;
    float respawn_delay;
    float bump_cooldown_time;
    float boost_pad_cooldown_big;
    float boost_pad_cooldown_small;
    float car_spawn_boost_amount;
    float ball_hit_extra_force_scale;
    float bump_force_scale;
    float ball_radius;
    uint8_t unlimited_flips;
    uint8_t unlimited_double_jumps;
    uint8_t recharge_boost_enabled;
    uint8_t _pad0;
    float recharge_boost_per_second;
    float recharge_boost_delay;
    uint8_t demo_mode;
    uint8_t enable_team_demos;
    uint8_t _pad1[2];
    float goal_base_threshold_y;
} rsg_mutator_config;

/* Event kinds delivered to the callbacks after a step completes. */
#define RSG_EVENT_GOAL 1      /* a = scoring team (Arena.cpp:748-752) */
#define RSG_EVENT_BUMP 2      /* a = bumper id, b = victim id, flag = is_demo (Arena.cpp:399-400) */
#define RSG_EVENT_BALL_HIT 3  /* a = car id; the reference records it in CarState::ballHitInfo (Ball.cpp:251-259) */

typedef struct rsg_event {
    uint32_t arena;
    uint32_t kind;
    uint64_t tick;
    uint32_t a;
    uint32_t b;
    uint32_t flag;
    uint32_t _pad0;
} rsg_event;

typedef struct rsg_batch rsg_batch;

/* Arena::GoalScoreEventFn (src/Sim/Arena/Arena.h:24) and CarBumpEventFn (Arena.h:25)
 * become one event callback each; they run on the host after the step's device work. */
typedef void (*rsg_goal_fn)(rsg_batch* batch, uint32_t arena, int scoring_team, void* user);
typedef void (*rsg_bump_fn)(rsg_batch* batch, uint32_t arena, uint32_t bumper_id, uint32_t victim_id,
                            int is_demo, void* user);
typedef void (*rsg_ball_hit_fn)(rsg_batch* batch, uint32_t arena, uint32_t car_id, uint64_t tick, void* user);

/* ---- lifecycle ------------------------------------------------------------ */

/* RocketSim::InitFromMem (src/RocketSim.h:27-32, src/RocketSim.cpp:98-185):
 * loads .cmf collision meshes (src/CollisionMeshFile/CollisionMeshFile.cpp:11-61)
 * for one game mode and builds the shared BVH used by every batch.
 * Idempotent per game mode like the reference (RocketSim.cpp:100-105). */
int rsg_init_from_mem(int game_mode, const uint8_t* const* mesh_files, const uint64_t* mesh_sizes,
                      int n_files);

/* Message of the last failing call on this thread (replaces RS_ERR_CLOSE). */
int rsg_get_last_error(char* buf, uint64_t buf_len);

/* Car preset lookup, CAR_CONFIG_* constants (CarConfig.cpp:94-100). */
int rsg_get_car_config_preset(int preset, rsg_car_config* out);

/* Arena::Create (src/Sim/Arena/Arena.h:111, Arena.cpp:416-544), batched:
 * n_arenas independent arenas of one game mode, each holding up to
 * max_cars_per_arena cars.  tick_rate must be 15..120 (Arena.cpp:419).
 * Allocates all device memory of the batch. */
rsg_batch* rsg_batch_create(int game_mode, uint32_t n_arenas, uint32_t max_cars_per_arena, float tick_rate);
/* rsg_batch_create with an ArenaConfig (Arena::Create's second argument,
 * Arena.h:111): custom boost pads (checked against every car without
 * BoostPadGrid, Arena.cpp:501-506, 724-728) and noBallRot. */
rsg_batch* rsg_batch_create_ex(int game_mode, uint32_t n_arenas, uint32_t max_cars_per_arena, float tick_rate,
                               const rsg_arena_config* config);
/* ArenaConfig's defaults */
int rsg_get_default_arena_config(rsg_arena_config* out);
void rsg_batch_destroy(rsg_batch* batch);
int rsg_batch_num_arenas(const rsg_batch* batch, uint32_t* out);
/* Boost pads per arena (Arena::GetBoostPads().size()): the pad arrays of the
 * state calls hold this many pads per arena. */
int rsg_batch_num_pads(const rsg_batch* batch, uint32_t* out);

/* MutatorConfig(GameMode) (MutatorConfig.cpp:5-40): the defaults of a game mode. */
int rsg_get_default_mutator_config(int game_mode, rsg_mutator_config* out);
/* Arena::SetMutatorConfig / GetMutatorConfig (Arena.cpp:17-48, Arena.h:52-53),
 * for every arena of the batch.  Cars added afterwards respawn with
 * car_spawn_boost_amount (Arena.cpp:58-59).  car_mass must stay at its default
 * (CAR_MASS_BT = 180): the reference applies a changed car mass
 * only to the cars that exist at the call, with the ball's mass
 * (Arena.cpp:35-41), and not to cars added later (Car.cpp:206-209); any other
 * value returns RSG_ERR_ARG.  Flows between ticks (synchronous). */
int rsg_set_mutator_config(rsg_batch* batch, const rsg_mutator_config* config);
int rsg_get_mutator_config(const rsg_batch* batch, rsg_mutator_config* out);

/* ---- cars ----------------------------------------------------------------- */

/* Arena::AddCar (Arena.h:71, Arena.cpp:50-62).  The car is placed with
 * Car::Respawn's state (Car.cpp:43-56) at respawn location `respawn_index`
 * (0..3); the reference draws that index from a time-seeded RNG, so callers
 * that need reproducibility pass it explicitly (or -1 for index 0). */
int rsg_add_car(rsg_batch* batch, uint32_t arena, int team, const rsg_car_config* config,
                int respawn_index, uint32_t* out_car_id);
/* Arena::RemoveCar(id) (Arena.h:74-80, Arena.cpp:80-94) */
int rsg_remove_car(rsg_batch* batch, uint32_t arena, uint32_t car_id);
/* Arena::GetCars (Arena.h:66): ids in the order per-car updates run. */
int rsg_get_car_ids(const rsg_batch* batch, uint32_t arena, uint32_t* out_ids, uint32_t cap, uint32_t* out_n);
/* The reference iterates its cars in std::unordered_set<Car*> order
 * (Arena.h:35, Arena.cpp:706,720), which depends on heap addresses.  This sets
 * the per-car update order explicitly (a permutation of the arena's car ids). */
int rsg_set_car_update_order(rsg_batch* batch, uint32_t arena, const uint32_t* ids, uint32_t n);

/* Writing Car::controls (Car.h:149); the reference has no setter. */
int rsg_set_car_controls(rsg_batch* batch, uint32_t arena, uint32_t car_id, const rsg_car_controls* controls);
/* Controls of every car slot of every arena from host memory, layout [arena][slot]
 * with max_cars_per_arena slots per arena (slot order == rsg_get_car_ids order). */
int rsg_set_controls_all(rsg_batch* batch, const rsg_car_controls* controls, uint64_t count);

/* Car::GetState / Car::SetState (Car.cpp:10-36) */
int rsg_get_car_state(rsg_batch* batch, uint32_t arena, uint32_t car_id, rsg_car_state* out);
int rsg_set_car_state(rsg_batch* batch, uint32_t arena, uint32_t car_id, const rsg_car_state* state);
/* Car::Demolish (Car.cpp:38-41) */
int rsg_demolish_car(rsg_batch* batch, uint32_t arena, uint32_t car_id, float respawn_delay);

/* ---- ball, pads, arena ---------------------------------------------------- */

/* Ball::GetState / Ball::SetState (Ball.cpp:27-51) */
int rsg_get_ball_state(rsg_batch* batch, uint32_t arena, rsg_ball_state* out);
int rsg_set_ball_state(rsg_batch* batch, uint32_t arena, const rsg_ball_state* state);
/* BallState::hsInfo (Ball.h:24-32), the heatseeker part of GetState / SetState: rsg_set_ball_state
 * resets it to a default BallState's (no target, 2900 uu/s, 0 s), as Ball::SetState does with a
 * fresh state; set it afterwards to carry it over.  Soccar arenas keep the default. */
int rsg_get_ball_heatseeker(rsg_batch* batch, uint32_t arena, rsg_heatseeker_info* out);
int rsg_set_ball_heatseeker(rsg_batch* batch, uint32_t arena, const rsg_heatseeker_info* in);
/* BoostPad::GetState / SetState (BoostPad.h:44-45); pad order of Arena.cpp:514-531 */
int rsg_get_pad_state(rsg_batch* batch, uint32_t arena, uint32_t pad, rsg_pad_state* out);
int rsg_set_pad_state(rsg_batch* batch, uint32_t arena, uint32_t pad, const rsg_pad_state* state);
/* BoostPadConfig of pad `pad` (BoostPad.h:14-18) */
int rsg_get_pad_config(const rsg_batch* batch, uint32_t pad, rsg_vec3* pos, int* is_big);
/* Arena::tickCount (Arena.h:64) */
int rsg_get_tick_count(rsg_batch* batch, uint32_t arena, uint64_t* out);
int rsg_set_tick_count(rsg_batch* batch, uint32_t arena, uint64_t tick_count);
/* Arena::IsBallScored (Arena.cpp:893-927) */
int rsg_is_ball_scored(rsg_batch* batch, uint32_t arena, int* out);

/* Bulk state transfer of the whole batch to / from host memory.  Car arrays are
 * [arena][slot] with max_cars_per_arena slots; empty slots are left untouched
 * on get and ignored on set.  Pads are [arena][34]. */
int rsg_get_all_states(rsg_batch* batch, rsg_car_state* cars, rsg_ball_state* balls, rsg_pad_state* pads);
int rsg_set_all_states(rsg_batch* batch, const rsg_car_state* cars, const rsg_ball_state* balls,
                       const rsg_pad_state* pads);

/* ---- stepping ------------------------------------------------------------- */

/* Arena::Step(ticks) (Arena.h:132, Arena.cpp:689-756) for every arena of the
 * batch.  Synchronous: returns after the device work is done and the event
 * callbacks have run. */
int rsg_step(rsg_batch* batch, int ticks);

/* Arena::Step one tick at a time with each car's controls set before every
 * tick (Car::controls, Car.h:149, read by Car::_PreTickUpdate), for every arena
 * of the batch: controls (host memory, pinned or not) holds [ticks][arena][slot]
 * controls, copied to the device at the call.  Synchronous like rsg_step. */
int rsg_step_controls(rsg_batch* batch, const rsg_car_controls* controls, int ticks);

/* Asynchronous variant on the batch's own stream for callers that keep
 * inputs resident in device memory: d_controls (device pointer, may be NULL
 * to keep the current controls) holds [ticks][arena][slot] controls.  Events
 * are queued on the device and delivered by the next rsg_sync(). */
int rsg_step_async(rsg_batch* batch, const rsg_car_controls* d_controls, int ticks);
int rsg_sync(rsg_batch* batch);
/* CUDA stream (cudaStream_t) the batch launches on, as void*. */
void* rsg_batch_stream(rsg_batch* batch);

/* Arena::SetGoalScoreCallback / SetCarBumpCallback (Arena.h:98-108), and a
 * ball-hit callback the reference does not have (it only records the hit in
 * CarState::ballHitInfo, Ball.cpp:251-259). */
int rsg_set_goal_callback(rsg_batch* batch, rsg_goal_fn fn, void* user);
int rsg_set_bump_callback(rsg_batch* batch, rsg_bump_fn fn, void* user);
int rsg_set_ball_hit_callback(rsg_batch* batch, rsg_ball_hit_fn fn, void* user);

/* ---- differentiable air-phase rollouts ------------------------------------ */

/* Contact-free rollouts of one car and the ball per instance, and their
 * adjoint.  No counterpart in the reference: they restate the air path of
 * Arena::Step (Car::_UpdateAirTorque, Car.cpp:584-669; the boost force of
 * Car::_UpdateBoost, Car.cpp:486-533, with the boost input relaxed to [0, 1];
 * gravity; btTransformUtil::integrateTransform, btTransformUtil.h:37-80; the
 * clamps of Car::_FinishPhysicsTick, Car.cpp:165-193; ball drag and clamps,
 * Ball.cpp:117-143) for gradient-based control.  For boost inputs of exactly
 * 0 or 1 held over the rollout the forward equals rsg_step on an airborne car
 * that touches nothing.
 *
 * All pointers are device pointers.  State: [n][24] floats per instance, Bullet
 * units: car position, velocity, angular velocity, basis rows (9), ball
 * position, ball velocity.  Controls: [ticks][n][4] = pitch, yaw, roll in
 * [-1, 1] and boost in [0, 1].  d_ckpt (may be NULL in the forward) receives
 * the state every ckpt_every (>= 1) ticks, [ceil(ticks / ckpt_every)][n][24];
 * the backward recomputes all segments from it at once.  d_grad_final is the
 * gradient of a loss with respect to the final state ([n][24]),
 * d_grad_controls receives the gradient with respect to the controls
 * ([ticks][n][4]; an input outside its range gets 0, one on its boundary
 * passes the gradient) and d_grad_state0 (may be NULL) the gradient with
 * respect to the initial state ([n][24]).  The backward needs a device
 * workspace of rsg_air_backward_workspace_size bytes (152 bytes per instance
 * and tick; RSG_ERR_ARG if smaller).  `stream` is a cudaStream_t or NULL;
 * the calls are asynchronous on it. */
int rsg_air_forward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_state0,
                    const float* d_controls, float* d_final, float* d_ckpt, int ckpt_every, void* stream);
int rsg_air_backward_workspace_size(int n, int ticks, size_t* bytes);
int rsg_air_backward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_controls,
                     const float* d_ckpt, int ckpt_every, const float* d_grad_final, float* d_grad_controls,
                     float* d_grad_state0, void* d_workspace, size_t workspace_bytes, void* stream);

/* rsg_air_backward for callers that cannot allocate device memory (a plugin
 * whose host program owns the device memory through its own allocator, or a
 * control loop that cannot afford the synchronisation cudaMalloc/cudaFree may
 * cause).  No counterpart in the reference.  Same arguments and results as
 * rsg_air_backward without the workspace: the tape lives in a 16 MiB static
 * device array, so n * ticks must be at most 110376 (RSG_ERR_ARG with a
 * message otherwise, nothing launched).  All calls on a device share that
 * array: calls whose kernels overlap on the GPU race, so order them on one
 * stream.  Nothing in it must start at zero.  The first call on each device
 * looks up the array's address (with that device current); make it before any
 * stream capture. */
int rsg_air_backward_noalloc(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_controls,
                             const float* d_ckpt, int ckpt_every, const float* d_grad_final, float* d_grad_controls,
                             float* d_grad_state0, void* stream);

/* ---- differentiable ground-driving rollouts -------------------------------- */

/* Rollouts of one car driving on the arena floor (z = 0) and the ball per
 * instance, and their adjoint.  No counterpart in the reference: they restate
 * the ground path of Arena::Step for a car with four wheels on the floor and a
 * chassis that touches nothing (btVehicleRL::rayCast, calcFrictionImpulses,
 * updateSuspension, applyFrictionImpulses, btVehicleRL.cpp:66-395;
 * Car::_UpdateWheels, Car.cpp:339-484, without handbrake; the ground boost
 * force of Car::_UpdateBoost, Car.cpp:486-533, with the boost input relaxed to
 * [0, 1] and its full throttle to throttle + boost (1 - throttle); gravity,
 * integrateTransform and the clamps of Car::_FinishPhysicsTick) for
 * gradient-based control.  For boost inputs of exactly 0 or 1 held over the
 * rollout the forward follows rsg_step on a car driving on the floor.
 *
 * All pointers are device pointers.  State: [n][39] floats per instance, Bullet
 * units: car position, velocity, angular velocity, basis rows (9), front steer
 * angle, engine force, brake force, lateral friction factor per wheel (4),
 * longitudinal friction factor per wheel (4), extra push-back per wheel (4),
 * ball position, ball velocity.  Controls: [ticks][n][4] = throttle and steer
 * in [-1, 1], boost in [0, 1], one unused float.  d_flags (may be NULL)
 * receives per instance the OR over the ticks of bit 0 (a wheel's ray missed
 * the floor) and bit 1 (the car tilted past the suspension's contact limit),
 * the ticks that left the model.  Checkpoints, gradients and workspace as for
 * the air rollouts, with 39 floats per state: the workspace is
 * rsg_ground_backward_workspace_size bytes (180 bytes per instance and tick).
 * The gradient at boost 1 is the one-sided derivative from inside [0, 1]. */
int rsg_ground_forward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_state0,
                       const float* d_controls, float* d_final, float* d_ckpt, int ckpt_every, int* d_flags,
                       void* stream);
int rsg_ground_backward_workspace_size(int n, int ticks, size_t* bytes);
int rsg_ground_backward(const rsg_car_config* car, float tick_rate, int n, int ticks, const float* d_controls,
                        const float* d_ckpt, int ckpt_every, const float* d_grad_final, float* d_grad_controls,
                        float* d_grad_state0, void* d_workspace, size_t workspace_bytes, void* stream);

/* ---- serialisation -------------------------------------------------------- */

/* Arena::Serialize (src/Sim/Arena/Arena.cpp:546-574) of arena `arena`, in
 * RocketSim's byte format (DataStreamOut, without the file's version word):
 * the reference's DeserializeNew reads it and rsg_deserialize_arena reads the
 * reference's output.  Cars are written by ascending id (the reference's
 * DeserializeNew keeps every car only then, Arena.cpp:590-606).  With
 * `out` NULL only *len is set; with `cap` < *len, RSG_ERR_ARG. */
int rsg_serialize_arena(rsg_batch* batch, uint32_t arena, uint8_t* out, uint64_t cap, uint64_t* len);
/* Arena::DeserializeNew (Arena.cpp:576-643) into arena `arena`: its cars are
 * replaced by the serialized ones (ids, teams, configurations, controls,
 * states), then the pads, the ball, the tick count and the last car id.  The
 * game mode, tick rate and arena config must be the batch's; mutators that
 * differ from the batch's are applied when the batch holds one arena.  As in
 * the reference, every car's boost comes back as the game mode's default spawn
 * amount (DeserializeNewCar sets up the car body after reading its state,
 * Arena.cpp:676-687 and Car.cpp:291); rsg_clone_arena keeps the boost. */
int rsg_deserialize_arena(rsg_batch* batch, uint32_t arena, const uint8_t* data, uint64_t len);
/* Arena::Clone (Arena.cpp:646-674): arena `src_arena` of `src` into arena
 * `dst_arena` of `dst` (callbacks stay with each batch). */
int rsg_clone_arena(rsg_batch* dst, uint32_t dst_arena, rsg_batch* src, uint32_t src_arena);

/* ---- kickoffs and goal prediction -------------------------------------------- */

/* Arena::ResetToRandomKickoff(seed) (src/Sim/Arena/Arena.cpp:113-222), soccar:
 * the kickoff spots shuffled by std::default_random_engine(seed) as libstdc++'s
 * std::shuffle does (seed -1: one engine for the process, seeded from the
 * clock), cars placed in update order, the ball at rest at the centre, every
 * pad reset.  The _many form resets arenas[k] with seeds[k] (seeds NULL: all
 * -1) in one transfer. */
int rsg_reset_to_random_kickoff(rsg_batch* batch, uint32_t arena, int32_t seed);
int rsg_reset_to_random_kickoff_many(rsg_batch* batch, const uint32_t* arenas, const int32_t* seeds, uint32_t n);
/* Arena::IsBallProbablyGoingIn(maxTime, extraMargin, &team) (Arena.cpp:770-806,
 * soccar) of every arena: out[n_arenas] 0/1, goal_team[n_arenas] (may be NULL)
 * the team whose goal line the ball crosses (RSG_TEAM_*; -1 where out is 0).
 * RSG_ERR_STATE for other game modes (the reference refuses them). */
int rsg_is_ball_probably_going_in(rsg_batch* batch, float max_time, float extra_margin, int* out, int* goal_team);

/* ---- game events ------------------------------------------------------------ */

/* GameEventTrackerConfig (src/Sim/GameEventTracker/GameEventTracker.h:10-40) and
 * its autoStateSetDetection flag (GameEventTracker.h:93). */
typedef struct rsg_game_event_tracker_config {
    float shot_min_speed;
    float shot_touch_min_delay;
    float pred_score_extra_margin;
    float shot_event_cooldown;
    float shot_min_score_time;
    float goal_max_touch_time;
    float pass_max_touch_time;
    uint8_t auto_state_set_detection;
    uint8_t _pad0[3];
} rsg_game_event_tracker_config;

#define RSG_GAME_EVENT_NONE 0
#define RSG_GAME_EVENT_SHOT 1 /* car_id: shooter, other_car_id: passer (0: none) */
#define RSG_GAME_EVENT_GOAL 2 /* car_id: scorer, other_car_id: passer (0: none) */
#define RSG_GAME_EVENT_SAVE 3 /* car_id: saver */
typedef struct rsg_game_event {
    int32_t kind;
    uint32_t car_id;
    uint32_t other_car_id;
} rsg_game_event;

/* GameEventTracker for every arena of a batch (soccar): Update() of all arenas
 * at once reports at most one event per arena (the reference's callbacks fire
 * at most once per Update). */
typedef struct rsg_game_event_tracker rsg_game_event_tracker;
int rsg_get_default_game_event_tracker_config(rsg_game_event_tracker_config* out);
rsg_game_event_tracker* rsg_game_event_tracker_create(rsg_batch* batch, const rsg_game_event_tracker_config* config);
void rsg_game_event_tracker_destroy(rsg_game_event_tracker* tracker);
/* GameEventTracker::Update (GameEventTracker.cpp:48-158) of every arena:
 * events[n_arenas] (host) receives each arena's event (kind RSG_GAME_EVENT_NONE if
 * none). */
int rsg_game_event_tracker_update(rsg_game_event_tracker* tracker, rsg_batch* batch, rsg_game_event* events);
/* ResetPersistentInfo (GameEventTracker.cpp:160-166) of one arena, or of all
 * with arena = -1. */
int rsg_game_event_tracker_reset_persistent_info(rsg_game_event_tracker* tracker, int32_t arena);

/* ---- ball prediction ------------------------------------------------------ */

/* BallPredTracker (src/Sim/BallPredTracker/BallPredTracker.h:7-35) for every
 * arena of a batch.  Each arena gets a ball-only shadow arena (the source's
 * game mode, arena config and tick rate; default mutators; no cars) and
 * `num_pred_ticks` predicted ball states (predData) in device memory.
 * Creation runs the constructor's UpdatePredFromArena (a full prediction from
 * the arenas' balls).  Update calls return when the predictions are written. */
typedef struct rsg_ball_pred rsg_ball_pred;
rsg_ball_pred* rsg_ball_pred_create(rsg_batch* batch, uint32_t num_pred_ticks);
void rsg_ball_pred_destroy(rsg_ball_pred* tracker);
/* UpdatePredFromArena (BallPredTracker.cpp:18-24) for every arena with
 * mask[a] != 0 (mask NULL: all): the batch's ball states and tick counts.
 * `batch` has the tracker's arena count; work queued on its stream comes
 * first. */
int rsg_ball_pred_update_from_batch(rsg_ball_pred* tracker, rsg_batch* batch, const uint8_t* mask);
/* UpdatePredManual (BallPredTracker.cpp:26-62): host arrays [n_arenas] of
 * current ball states and ticks since the last update.  With 0 <= k <
 * num_pred_ticks and predData[k] matching the current state (BallState::
 * Matches, Ball.cpp:12-17) the prediction is shifted by k and extended by k
 * ticks; otherwise everything is predicted again. */
int rsg_ball_pred_update_manual(rsg_ball_pred* tracker, const rsg_ball_state* cur,
                                const int32_t* ticks_since_last_update, const uint8_t* mask);
/* ForceUpdateAllPred (BallPredTracker.cpp:64-72) from initial[n_arenas]. */
int rsg_ball_pred_force_update_all(rsg_ball_pred* tracker, const rsg_ball_state* initial, const uint8_t* mask);
uint32_t rsg_ball_pred_num_pred_ticks(const rsg_ball_pred* tracker);
/* predData of one arena, front first: out[num_pred_ticks]. */
int rsg_ball_pred_get_pred(rsg_ball_pred* tracker, uint32_t arena, rsg_ball_state* out);
/* predData of every arena: out[n_arenas][num_pred_ticks], front first. */
int rsg_ball_pred_get_all(rsg_ball_pred* tracker, rsg_ball_state* out);
/* GetBallStateForTime (BallPredTracker.cpp:74-79). */
int rsg_ball_pred_get_state_for_time(rsg_ball_pred* tracker, uint32_t arena, float pred_time, rsg_ball_state* out);
/* lastUpdateTickCount (BallPredTracker.h:12) of one arena. */
int rsg_ball_pred_get_last_update_tick(rsg_ball_pred* tracker, uint32_t arena, int32_t* out);
/* The device ring: d_pred[a * num_pred_ticks + (d_head[a] + i) % num_pred_ticks]
 * is predData[i] of arena a (valid between update calls). */
int rsg_ball_pred_device_buffers(rsg_ball_pred* tracker, const rsg_ball_state** d_pred, const uint32_t** d_head);
/* Device error flags of the shadow arenas ([n_arenas] words, as rsg_get_device_flags). */
int rsg_ball_pred_device_flags(rsg_ball_pred* tracker, uint32_t* out);

/* Device flags of every arena after the last step ([n_arenas] words).  Bits 0-7
 * are errors (the step also returns RSG_ERR_DEVICE): bits 0-3 capacity
 * overflows, bit 4 a non-finite state, bit 5 a tick launch wider than the
 * batch's scratch (the arena was not stepped; the host never launches one); bit 8 marks a
 * box contact deeper than GJK resolves and bit 9 overlapping car boxes, two
 * contact kinds the restated narrow phase does not produce yet.  No counterpart
 * in the reference. */
int rsg_get_device_flags(rsg_batch* batch, uint32_t* out);

/* Launch shape of the batch's tick kernel: out[0] arenas per block, out[1] threads
 * per car in the vehicle update, out[2] BVH subtree headers in shared memory (1) or
 * read through L2 (0; -1 automatic), out[3] wheel rays on the leaf grid (1) or
 * walking the BVH (0), out[4] block-wide barriers between the parts of the collision
 * work (1) or not (0), out[5] a persistent launch (as many blocks as are resident,
 * each taking groups of arenas from a device counter, 1) or one block per group (0).
 * Chosen by the tuner on the batch's first launch (every shape gives the same
 * results) or fixed by the environment variable RSG_TICK_SHAPE (the numbers comma
 * separated, the last two optional).  No counterpart in the reference. */
int rsg_get_tick_shape(const rsg_batch* batch, int32_t out[6]);
/* The tuner's trials as text (shapes and milliseconds per tick), NUL-terminated and
 * cut to buf_len.  No counterpart in the reference. */
int rsg_get_tuning_log(const rsg_batch* batch, char* buf, uint64_t buf_len);

#ifdef __cplusplus
}
#endif

#endif /* ROCKETSIM_GB300_H */
