// rsg_mesh.h -- arena collision mesh: .cmf parsing, quantized BVH, internal-edge
// info and broadphase cell map, built once on the host and uploaded to the GPU.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "rsg_math.cuh"

namespace rsg {

// 16-byte quantized BVH node (B/BulletCollision/BroadphaseCollision/btQuantizedBvh.h:52-90)
struct QNode {
    uint16_t qmin[3], qmax[3];
    int32_t esc_or_tri;  // >= 0: triangle index (leaf); < 0: -escape index
};
struct Subtree {  // btBvhSubtreeInfo
    uint16_t qmin[3], qmax[3];
    int32_t root, size;
};
struct TriInfo {  // btTriangleInfo; present == 0 when the triangle has no shared edge
    int32_t flags;
    float a01, a12, a20;
    int32_t present;
};
enum : int32_t {
    TRI_V0V1_CONVEX = 1, TRI_V1V2_CONVEX = 2, TRI_V2V0_CONVEX = 4,
    TRI_V0V1_SWAP = 8, TRI_V1V2_SWAP = 16, TRI_V2V0_SWAP = 32
};

// Broadphase voxel grid of RocketSim's default ArenaConfig
// (src/Sim/Arena/ArenaConfig/ArenaConfig.h:25-33, btRSBroadphase.cpp:35-60)
struct GridSpec {
    V3 mn, mx;
    float cell;
    int nx, ny, nz;
};
GridSpec default_grid();

struct HostMesh {
    int ntri = 0;
    std::vector<V3> tri_verts;  // 3 per triangle
    V3 aabb_min, aabb_max;       // local AABB, margin 0
    V3 bvh_min, bvh_max, quant;
    std::vector<QNode> nodes;
    int cur_node = 0;
    std::vector<Subtree> subtrees;
    std::vector<QNode> sub_groups;  // quantized box around each run of 32 subtree headers
    std::vector<TriInfo> info;
    std::vector<uint8_t> mesh_cells;  // broadphase cells where the mesh proxy is registered
    // Leaf grid: a uniform grid over the BVH's quantized space (cell = quantized coordinate >>
    // lg_shift per axis) listing, per cell and in node order, the leaf nodes whose quantized box
    // touches the cell.  A query box's leaves are then found without walking the tree.
    // Each cell is a 64-byte block: a header (leaf count, offset of the leaves past the first three
    // in lg_over) and the first three leaf records.  A record is the leaf's quantized box with
    // esc_or_tri = (the leaf's rank in node order << 16) | its triangle index.  Empty when the mesh
    // has more than 65535 triangles (queries then walk the tree).
    int lg_shift[3] = {0, 0, 0}, lg_n[3] = {0, 0, 0};
    std::vector<QNode> lg_block;  // 4 QNode-sized slots per cell: header, three records
    std::vector<QNode> lg_over;   // the remaining records of every cell, cell by cell
};

// Parses one .cmf file (src/CollisionMeshFile/CollisionMeshFile.cpp:11-61) and
// builds everything.  Returns false and fills `err` on malformed input.
bool build_mesh(const uint8_t* data, uint64_t len, HostMesh& out, std::string& err);

}  // namespace rsg
