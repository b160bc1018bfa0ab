// rs_oracle.h -- C API of the CPU restatement of RocketSim's Arena::Step.
//
// TEST ORACLE ONLY.  This library is the checker for the CUDA path: tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the
// product never links or calls it.  Its surface mirrors oracle/ref_driver.cpp
// (prefix rsora_ instead of rsref_) so one Python harness drives either.
#pragma once
#include <stdint.h>
#include "../include/rocketsim_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int rsora_init(const uint8_t* cmf, uint64_t len);
void* rsora_arena_create(int game_mode, float tick_rate);
void rsora_arena_destroy(void* h);
int rsora_preset(int preset, rsg_car_config* out);
uint32_t rsora_add_car(void* h, int team, int preset);
int rsora_car_order(void* h, uint32_t* out, uint32_t cap);
int rsora_set_car_order(void* h, const uint32_t* ids, uint32_t n);
int rsora_set_controls(void* h, uint32_t id, const rsg_car_controls* c);
int rsora_get_car(void* h, uint32_t id, rsg_car_state* out);
int rsora_set_car(void* h, uint32_t id, const rsg_car_state* s);
int rsora_get_ball(void* h, rsg_ball_state* out);
int rsora_set_ball(void* h, const rsg_ball_state* in);
int rsora_num_pads(void* h);
int rsora_get_pad(void* h, int i, rsg_pad_state* out);
int rsora_set_pad(void* h, int i, const rsg_pad_state* in);
int rsora_pad_config(void* h, int i, rsg_vec3* pos, int* is_big);
uint64_t rsora_get_tick(void* h);
void rsora_set_tick(void* h, uint64_t t);
int rsora_step(void* h, int ticks);
int rsora_run(void* h, const rsg_car_controls* controls, int ncars, int ticks);
int rsora_is_scored(void* h);
int rsora_pop_events(void* h, uint64_t* out, int cap);
int rsora_get_wheel_internals(void* h, uint32_t id, float* out8);
// counters of narrow-phase paths taken (debug / coverage)
int rsora_get_counters(void* h, uint64_t* out, int cap);

#ifdef __cplusplus
}
#endif
