// rsg_view.cuh -- pieces shared by the translation units that run the arena tick: the kernel's
// view of a batch's buffers, and the conversions between an arena record and the public state
// structs (uu units, row-major basis in the record, forward / right / up columns in the structs).
#pragma once
#include "rsg_kernels.h"
#include "rsg_tick.cuh"

namespace rsg {

inline BatchView make_view(const BatchBuffers& b) {
    BatchView v;
    v.A = b.A;
    v.MC = b.MC;
    v.has_arena = b.has_arena;
    v.dt = b.dt;
    v.mut = b.mut;
    v.pad_cfg = b.pad_cfg;
    v.npads = b.npads;
    v.custom_pads = b.custom_pads;
    v.no_ball_rot = b.no_ball_rot;
    v.heatseeker = b.heatseeker;
    v.lanes_per_car = 4;
    v.rec = b.rec;
    v.rec_words = rec_words(b.MC);
    v.au = b.au;
    v.cfgs = b.cfgs;
    v.events = (DevEvent*)b.events;
    v.event_mask = b.event_mask;
    v.tick_scratch = b.tick_scratch;
    v.scratch_slots = b.scratch_slots;
    v.mesh.tv = b.mesh.tv;
    v.mesh.nodes = b.mesh.nodes;
    v.mesh.sub = b.mesh.sub;
    v.mesh.info = b.mesh.info;
    v.mesh.cells = b.mesh.cells;
    v.mesh.lg_block = b.mesh.lg_block;
    v.mesh.lg_over = b.mesh.lg_over;
    v.mesh.sub_grp = b.mesh.sub_grp;
    v.mesh.nsub_grp = b.mesh.nsub_grp;
    for (int k = 0; k < 3; k++) {
        v.mesh.lg_shift[k] = b.mesh.lg_shift[k];
        v.mesh.lg_n[k] = b.mesh.lg_n[k];
    }
    v.mesh.ntri = b.mesh.ntri;
    v.mesh.nnodes = b.mesh.nnodes;
    v.mesh.nsub = b.mesh.nsub;
    v.mesh.bvh_min = b.mesh.bvh_min;
    v.mesh.bvh_max = b.mesh.bvh_max;
    v.mesh.quant = b.mesh.quant;
    v.mesh.aabb_min = b.mesh.aabb_min;
    v.mesh.aabb_max = b.mesh.aabb_max;
    v.grid.mn = b.grid.mn;
    v.grid.cell = b.grid.cell;
    v.grid.nx = b.grid.nx;
    v.grid.ny = b.grid.ny;
    v.grid.nz = b.grid.nz;
    return v;
}

RSG_D rsg_vec3 to_rv(V3 v) { rsg_vec3 r; r.x = v.x; r.y = v.y; r.z = v.z; return r; }
RSG_D V3 from_rv(const rsg_vec3& v) { return V3(v.x, v.y, v.z); }
RSG_D M3 rot_to_basis(const rsg_rotmat& r) {  // columns forward / right / up
    return M3(r.forward.x, r.right.x, r.up.x, r.forward.y, r.right.y, r.up.y, r.forward.z, r.right.z, r.up.z);
}
RSG_D rsg_rotmat basis_to_rot(const M3& m) {
    rsg_rotmat r;
    r.forward = to_rv(m.col(0));
    r.right = to_rv(m.col(1));
    r.up = to_rv(m.col(2));
    return r;
}
RSG_D uint64_t u64(uint32_t lo, uint32_t hi) { return (uint64_t)lo | ((uint64_t)hi << 32); }

// Ball::GetState (src/Sim/Ball/Ball.cpp:27-33) from an arena record
RSG_D rsg_ball_state ball_get(const SoA& s) {
    rsg_ball_state o;
    o.pos = to_rv(V3(s.bf(BF_POS), s.bf(BF_POS + 1), s.bf(BF_POS + 2)) * RL::BT_TO_UU);
    M3 m;
    for (int r = 0; r < 3; r++) m.r[r] = V3(s.bf(BF_BASIS + 3 * r), s.bf(BF_BASIS + 3 * r + 1), s.bf(BF_BASIS + 3 * r + 2));
    o.rot_mat = basis_to_rot(m);
    o.vel = to_rv(V3(s.bf(BF_VEL), s.bf(BF_VEL + 1), s.bf(BF_VEL + 2)) * RL::BT_TO_UU);
    o.ang_vel = to_rv(V3(s.bf(BF_ANG), s.bf(BF_ANG + 1), s.bf(BF_ANG + 2)));
    o.tick_count_since_update = u64(s.bu(BU_TICKS_LO), s.bu(BU_TICKS_HI));
    return o;
}

// Ball::SetState (src/Sim/Ball/Ball.cpp:35-51) into an arena record
RSG_D void ball_set(const SoA& s, const rsg_ball_state& st) {
    V3 p = from_rv(st.pos) * RL::UU_TO_BT, v = from_rv(st.vel) * RL::UU_TO_BT;
    M3 m = rot_to_basis(st.rot_mat);
    s.bf(BF_POS) = p.x; s.bf(BF_POS + 1) = p.y; s.bf(BF_POS + 2) = p.z;
    for (int r = 0; r < 3; r++) {
        s.bf(BF_BASIS + 3 * r) = m.r[r].x;
        s.bf(BF_BASIS + 3 * r + 1) = m.r[r].y;
        s.bf(BF_BASIS + 3 * r + 2) = m.r[r].z;
    }
    s.bf(BF_VEL) = v.x; s.bf(BF_VEL + 1) = v.y; s.bf(BF_VEL + 2) = v.z;
    s.bf(BF_ANG) = st.ang_vel.x; s.bf(BF_ANG + 1) = st.ang_vel.y; s.bf(BF_ANG + 2) = st.ang_vel.z;
    // a default BallState's HeatseekerInfo (Ball.h:24-32)
    s.bf(BF_HS_DIR) = 0.f;
    s.bf(BF_HS_SPEED) = RL::HS::INITIAL_TARGET_SPEED;
    s.bf(BF_HS_TIME) = 0.f;
    s.bu(BU_TICKS_LO) = 0;
    s.bu(BU_TICKS_HI) = 0;
}

}  // namespace rsg
