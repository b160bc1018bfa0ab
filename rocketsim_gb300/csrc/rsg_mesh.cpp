// rsg_mesh.cpp -- host-side construction of the arena mesh acceleration data.
//
// The BVH is built with the same splitting rules, quantization and subtree
// headers as Bullet's btQuantizedBvh (B/BulletCollision/BroadphaseCollision/
// btQuantizedBvh.cpp:70-330, B/BulletCollision/CollisionShapes/
// btOptimizedBvh.cpp:23-140), because the order in which a query visits
// triangles decides the order of contact points in a manifold and therefore the
// solver result.  Internal-edge angles follow btGenerateInternalEdgeInfo
// (B/BulletCollision/CollisionDispatch/btInternalEdgeUtility.cpp:33-305).
#include "rsg_mesh.h"

#include <algorithm>
#include <cstring>

namespace rsg {

GridSpec default_grid() {
    const float UU_TO_BT = 1.f / 50.f;
    GridSpec g;
    g.mn = V3(-5600, -6000, 0) * UU_TO_BT;
    g.mx = V3(5600, 6000, 2200) * UU_TO_BT;
    g.cell = 370 * UU_TO_BT;
    V3 r = g.mx - g.mn;
    g.nx = std::max(1, (int)std::ceil(r.x / g.cell));
    g.ny = std::max(1, (int)std::ceil(r.y / g.cell));
    g.nz = std::max(1, (int)std::ceil(r.z / g.cell));
    return g;
}

namespace {

struct Builder {
    HostMesh& m;
    std::vector<QNode> leaves;
    explicit Builder(HostMesh& mesh) : m(mesh) {}

    void quantize(uint16_t* out, V3 p, bool is_max) const {
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
    void quantize_clamp(uint16_t* out, V3 p, bool is_max) const {
        quantize(out, vmin(vmax(p, m.bvh_min), m.bvh_max), is_max);
    }
    V3 unquantize(const uint16_t* q) const {
        V3 o((float)q[0] / m.quant.x, (float)q[1] / m.quant.y, (float)q[2] / m.quant.z);
        return o + m.bvh_min;
    }
    void set_quantization(V3 mn, V3 mx) {
        V3 c(1.f, 1.f, 1.f);
        m.bvh_min = mn - c;
        m.bvh_max = mx + c;
        V3 size = m.bvh_max - m.bvh_min;
        m.quant = V3(65533.f / size.x, 65533.f / size.y, 65533.f / size.z);
        uint16_t q[3];
        quantize(q, m.bvh_min, false);
        m.bvh_min = vmin(m.bvh_min, unquantize(q) - c);
        size = m.bvh_max - m.bvh_min;
        m.quant = V3(65533.f / size.x, 65533.f / size.y, 65533.f / size.z);
        quantize(q, m.bvh_max, true);
        m.bvh_max = vmax(m.bvh_max, unquantize(q) + c);
        size = m.bvh_max - m.bvh_min;
        m.quant = V3(65533.f / size.x, 65533.f / size.y, 65533.f / size.z);
    }
    V3 lmin(int i) const { return unquantize(leaves[i].qmin); }
    V3 lmax(int i) const { return unquantize(leaves[i].qmax); }
    int split_axis(int s, int e) const {
        V3 means(0, 0, 0), var(0, 0, 0);
        int n = e - s;
        for (int i = s; i < e; i++) means += 0.5f * (lmax(i) + lmin(i));
        means *= (1.f / (float)n);
        for (int i = s; i < e; i++) {
            V3 d = 0.5f * (lmax(i) + lmin(i)) - means;
            var += d * d;
        }
        var *= (1.f / ((float)n - 1));
        return max_axis(var);
    }
    int sort_split(int s, int e, int axis) {
        int split = s, n = e - s;
        V3 means(0, 0, 0);
        for (int i = s; i < e; i++) means += 0.5f * (lmax(i) + lmin(i));
        means *= (1.f / (float)n);
        float sv = means[axis];
        for (int i = s; i < e; i++) {
            V3 c = 0.5f * (lmax(i) + lmin(i));
            if (c[axis] > sv) {
                std::swap(leaves[i], leaves[split]);
                split++;
            }
        }
        int rb = n / 3;
        if ((split <= (s + rb)) || (split >= (e - 1 - rb))) split = s + (n >> 1);
        return split;
    }
    void add_subtree(int idx) {
        const QNode& nd = m.nodes[idx];
        int sz = nd.esc_or_tri >= 0 ? 1 : -nd.esc_or_tri;
        if (sz * (int)sizeof(QNode) > 2048) return;
        Subtree st;
        std::memcpy(st.qmin, nd.qmin, 6);
        std::memcpy(st.qmax, nd.qmax, 6);
        st.root = idx;
        st.size = sz;
        m.subtrees.push_back(st);
    }
    void build(int s, int e) {
        int n = e - s;
        int cur = m.cur_node;
        if (n == 1) {
            m.nodes[m.cur_node++] = leaves[s];
            return;
        }
        int axis = split_axis(s, e);
        int split = sort_split(s, e, axis);
        int internal = m.cur_node;
        quantize(m.nodes[internal].qmin, m.bvh_max, false);
        quantize(m.nodes[internal].qmax, m.bvh_min, true);
        for (int i = s; i < e; i++) {
            uint16_t qa[3], qb[3];
            quantize(qa, lmin(i), false);
            quantize(qb, lmax(i), true);
            for (int k = 0; k < 3; k++) {
                if (m.nodes[internal].qmin[k] > qa[k]) m.nodes[internal].qmin[k] = qa[k];
                if (m.nodes[internal].qmax[k] < qb[k]) m.nodes[internal].qmax[k] = qb[k];
            }
        }
        m.cur_node++;
        int left = m.cur_node;
        build(s, split);
        int right = m.cur_node;
        build(split, e);
        int esc = m.cur_node - cur;
        if (esc * (int)sizeof(QNode) > 2048) {  // btQuantizedBvh::updateSubtreeHeaders
            add_subtree(left);
            add_subtree(right);
        }
        m.nodes[internal].esc_or_tri = -esc;
    }
    static bool qov(const uint16_t* a0, const uint16_t* a1, const uint16_t* b0, const uint16_t* b1) {
        bool o = true;
        o = (a0[0] > b1[0] || a1[0] < b0[0]) ? false : o;
        o = (a0[2] > b1[2] || a1[2] < b0[2]) ? false : o;
        o = (a0[1] > b1[1] || a1[1] < b0[1]) ? false : o;
        return o;
    }
    template <class F>
    void query(V3 mn, V3 mx, F&& f) const {
        uint16_t qa[3], qb[3];
        quantize_clamp(qa, mn, false);
        quantize_clamp(qb, mx, true);
        for (const Subtree& st : m.subtrees) {
            if (!qov(qa, qb, st.qmin, st.qmax)) continue;
            int cur = st.root, end = st.root + st.size;
            while (cur < end) {
                const QNode& nd = m.nodes[cur];
                bool ov = qov(qa, qb, nd.qmin, nd.qmax);
                bool leaf = nd.esc_or_tri >= 0;
                if (leaf && ov) f(nd.esc_or_tri);
                if (ov || leaf) cur++;
                else cur += -nd.esc_or_tri;
            }
        }
    }

    void edge_info() {
        m.info.assign(m.ntri, TriInfo{0, TWO_PI_F, TWO_PI_F, TWO_PI_F, 0});
        const float EQV = 0.0001f * 0.0001f, PLANAR = 0.0001f;
        for (int ta = 0; ta < m.ntri; ta++) {
            const V3* A = &m.tri_verts[ta * 3];
            V3 mn(BT_LARGE, BT_LARGE, BT_LARGE), mx(-BT_LARGE, -BT_LARGE, -BT_LARGE);
            for (int j = 0; j < 3; j++) { mn = vmin(mn, A[j]); mx = vmax(mx, A[j]); }
            query(mn, mx, [&](int tb) {
                if (tb == ta) return;
                const V3* B = &m.tri_verts[tb * 3];
                if (len2(cross(B[1] - B[0], B[2] - B[0])) < EQV) return;
                if (len2(cross(A[1] - A[0], A[2] - A[0])) < EQV) return;
                int ns = 0, sa[3] = {-1, -1, -1}, sb[3] = {-1, -1, -1};
                for (int i = 0; i < 3; i++) {
                    for (int j = 0; j < 3; j++)
                        if (len2(A[i] - B[j]) < EQV) {
                            sa[ns] = i; sb[ns] = j; ns++;
                            if (ns >= 3) return;
                        }
                    if (ns >= 3) return;
                }
                if (ns != 2) return;
                if (sa[0] == 0 && sa[1] == 2) {
                    sa[0] = 2; sa[1] = 0;
                    std::swap(sb[0], sb[1]);
                }
                TriInfo& inf = m.info[ta];
                inf.present = 1;
                int sumA = sa[0] + sa[1];
                int otherA = 3 - sumA;
                V3 edge = A[sa[1]] - A[sa[0]];
                int otherB = 3 - (sb[0] + sb[1]);
                V3 tB0 = B[sb[1]], tB1 = B[sb[0]], tB2 = B[otherB];
                V3 nA = normalized(cross(A[1] - A[0], A[2] - A[0]));
                V3 nB = normalized(cross(tB1 - tB0, tB2 - tB0));
                edge = normalized(edge);
                V3 ecA = normalized(cross(edge, nA));
                if (dot(ecA, A[otherA] - A[sa[0]]) < 0) ecA *= -1;
                V3 ecB = normalized(cross(edge, nB));
                if (dot(ecB, B[otherB] - B[sb[0]]) < 0) ecB *= -1;
                float corrected = 0;
                bool convex = false;
                V3 ce = cross(ecA, ecB);
                if (!(len2(ce) < PLANAR)) {
                    ce = normalized(ce);
                    V3 cnA = normalized(cross(ce, ecA));
                    float angle2 = std::atan2(dot(ecB, cnA), dot(ecB, ecA));
                    float ang4 = PI_F - angle2;
                    convex = dot(nA, ecB) < 0.f;
                    corrected = convex ? ang4 : -ang4;
                }
                V3 e;
                int32_t swapf, convf;
                float* ang;
                if (sumA == 1) { e = A[0] - A[1]; swapf = TRI_V0V1_SWAP; convf = TRI_V0V1_CONVEX; ang = &inf.a01; }
                else if (sumA == 2) { e = A[2] - A[0]; swapf = TRI_V2V0_SWAP; convf = TRI_V2V0_CONVEX; ang = &inf.a20; }
                else { e = A[1] - A[2]; swapf = TRI_V1V2_SWAP; convf = TRI_V1V2_CONVEX; ang = &inf.a12; }
                Q orn = q_axis_angle(e, -corrected);
                if (dot(q_rotate(orn, nA), nB) < 0) inf.flags |= swapf;
                *ang = -corrected;
                if (convex) inf.flags |= convf;
            });
        }
    }

    // _UpdateCellsStatic<true> for the triangle-mesh proxy (btRSBroadphase.cpp:71-140)
    void cells() {
        GridSpec g = default_grid();
        m.mesh_cells.assign((size_t)g.nx * g.ny * g.nz, 0);
        V3 lhe = 0.5f * (m.aabb_max - m.aabb_min), lc = 0.5f * (m.aabb_max + m.aabb_min);
        V3 amin = (lc - lhe) - V3(0.02f, 0.02f, 0.02f), amax = (lc + lhe) + V3(0.02f, 0.02f, 0.02f);
        for (int a = 0; a < 3; a++) amax[a] = std::min(amax[a], g.mx[a]);
        auto idx3 = [&](V3 p, int& i, int& j, int& k) {
            V3 f = (p - g.mn) / g.cell;
            i = std::min(std::max((int)f.x, 0), g.nx - 1);
            j = std::min(std::max((int)f.y, 0), g.ny - 1);
            k = std::min(std::max((int)f.z, 0), g.nz - 1);
        };
        int i0, j0, k0, i1, j1, k1;
        idx3(amin, i0, j0, k0);
        idx3(amax, i1, j1, k1);
        for (int i = i0; i <= i1; i++)
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++) {
                    V3 cmn = g.mn + V3((float)i, (float)j, (float)k) * g.cell;
                    V3 cmx = cmn + V3(g.cell, g.cell, g.cell);
                    bool hit = false;
                    query(cmn, cmx, [&](int) { hit = true; });
                    if (!hit) continue;
                    for (int a = -1; a <= 1; a++)
                        for (int b = -1; b <= 1; b++)
                            for (int c = -1; c <= 1; c++) {
                                int ci = i + a, cj = j + b, ck = k + c;
                                if (ci < 0 || cj < 0 || ck < 0 || ci >= g.nx || cj >= g.ny || ck >= g.nz) continue;
                                m.mesh_cells[(size_t)ci * g.ny * g.nz + cj * g.nz + ck] = 1;
                            }
                }
    }
};

}  // namespace

// Leaf grid over the quantized BVH space, cells of about RSG_LEAF_GRID_CELL Bullet units per axis
// (a power of two quanta, so a quantized coordinate's cell is a shift).
#ifndef RSG_LEAF_GRID_CELL
#define RSG_LEAF_GRID_CELL 2.5f
#endif
void build_leaf_grid(HostMesh& m) {
    m.lg_block.clear();
    m.lg_over.clear();
    if (m.ntri > 65535) return;
    for (int k = 0; k < 3; k++) {
        float quanta = RSG_LEAF_GRID_CELL * m.quant[k];
        int sh = 4;
        while (sh < 15 && (float)(1 << (sh + 1)) <= quanta * 1.41421356f) sh++;
        m.lg_shift[k] = sh;
        m.lg_n[k] = (65535 >> sh) + 1;
    }
    const size_t ncell = (size_t)m.lg_n[0] * m.lg_n[1] * m.lg_n[2];
    std::vector<std::vector<QNode>> cells(ncell);
    int rank = 0;
    for (int j = 0; j < m.cur_node; j++) {  // node order, so every cell's list is sorted
        if (m.nodes[j].esc_or_tri < 0) continue;
        QNode q = m.nodes[j];
        q.esc_or_tri = (int32_t)(((uint32_t)rank << 16) | (uint32_t)m.nodes[j].esc_or_tri);
        rank++;
        int c0[3], c1[3];
        for (int k = 0; k < 3; k++) { c0[k] = q.qmin[k] >> m.lg_shift[k]; c1[k] = q.qmax[k] >> m.lg_shift[k]; }
        for (int x = c0[0]; x <= c1[0]; x++)
            for (int y = c0[1]; y <= c1[1]; y++)
                for (int z = c0[2]; z <= c1[2]; z++) cells[((size_t)x * m.lg_n[1] + y) * m.lg_n[2] + z].push_back(q);
    }
    m.lg_block.assign(ncell * 4, QNode{});
    for (size_t c = 0; c < ncell; c++) {
        const std::vector<QNode>& v = cells[c];
        QNode& hdr = m.lg_block[c * 4];
        uint32_t words[4] = {(uint32_t)v.size(), (uint32_t)m.lg_over.size(), 0, 0};
        std::memcpy(&hdr, words, sizeof(words));
        for (size_t i = 0; i < v.size(); i++) {
            if (i < 3) m.lg_block[c * 4 + 1 + i] = v[i];
            else m.lg_over.push_back(v[i]);
        }
    }
}

bool build_mesh(const uint8_t* data, uint64_t len, HostMesh& m, std::string& err) {
    if (!data || len < 8) { err = "mesh file too short"; return false; }
    int32_t nt, nv;
    std::memcpy(&nt, data, 4);
    std::memcpy(&nv, data + 4, 4);
    if (std::min(nt, nv) <= 0 || std::max(nt, nv) > 1000000) { err = "bad triangle/vertex count"; return false; }
    uint64_t need = 8ull + (uint64_t)nt * 12 + (uint64_t)nv * 12;
    if (need > len) { err = "mesh data overflown"; return false; }
    std::vector<int32_t> idx((size_t)nt * 3);
    std::memcpy(idx.data(), data + 8, (size_t)nt * 12);
    std::vector<V3> verts(nv);
    const uint8_t* vp = data + 8 + (size_t)nt * 12;
    for (int i = 0; i < nv; i++) {
        float f[3];
        std::memcpy(f, vp + (size_t)i * 12, 12);
        verts[i] = V3(f[0], f[1], f[2]);
    }
    for (int32_t v : idx)
        if (v < 0 || v >= nv) { err = "bad triangle vertex index"; return false; }
    m.ntri = nt;
    m.tri_verts.resize((size_t)nt * 3);
    for (int i = 0; i < nt * 3; i++) m.tri_verts[i] = verts[idx[i]];
    V3 mn(BT_LARGE, BT_LARGE, BT_LARGE), mx(-BT_LARGE, -BT_LARGE, -BT_LARGE);
    for (const V3& v : m.tri_verts) { mn = vmin(mn, v); mx = vmax(mx, v); }
    m.aabb_min = mn;
    m.aabb_max = mx;
    Builder b(m);
    b.set_quantization(mn, mx);
    b.leaves.resize(nt);
    for (int t = 0; t < nt; t++) {
        V3 a(BT_LARGE, BT_LARGE, BT_LARGE), c(-BT_LARGE, -BT_LARGE, -BT_LARGE);
        for (int j = 0; j < 3; j++) { a = vmin(a, m.tri_verts[t * 3 + j]); c = vmax(c, m.tri_verts[t * 3 + j]); }
        for (int k = 0; k < 3; k++)
            if (c[k] - a[k] < 0.002f) { c[k] = c[k] + 0.001f; a[k] = a[k] - 0.001f; }
        b.quantize(b.leaves[t].qmin, a, false);
        b.quantize(b.leaves[t].qmax, c, true);
        b.leaves[t].esc_or_tri = t;
    }
    m.nodes.assign((size_t)2 * nt, QNode{});
    m.cur_node = 0;
    m.subtrees.clear();
    b.build(0, nt);
    if (m.subtrees.empty()) b.add_subtree(0);
    if (m.subtrees.empty()) {  // a single tree larger than one header still gets one
        Subtree st;
        std::memcpy(st.qmin, m.nodes[0].qmin, 6);
        std::memcpy(st.qmax, m.nodes[0].qmax, 6);
        st.root = 0;
        st.size = m.nodes[0].esc_or_tri >= 0 ? 1 : -m.nodes[0].esc_or_tri;
        m.subtrees.push_back(st);
    }
    m.nodes.resize(m.cur_node);
    b.edge_info();
    b.cells();
    build_leaf_grid(m);
    m.sub_groups.clear();
    for (size_t g = 0; g < m.subtrees.size(); g += 32) {
        QNode q{};
        for (int k = 0; k < 3; k++) { q.qmin[k] = 0xffff; q.qmax[k] = 0; }
        for (size_t h = g; h < m.subtrees.size() && h < g + 32; h++)
            for (int k = 0; k < 3; k++) {
                q.qmin[k] = std::min(q.qmin[k], m.subtrees[h].qmin[k]);
                q.qmax[k] = std::max(q.qmax[k], m.subtrees[h].qmax[k]);
            }
        q.esc_or_tri = (int32_t)g;
        m.sub_groups.push_back(q);
    }
    return true;
}

}  // namespace rsg
