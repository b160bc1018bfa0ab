// rsg_epa.cuh -- GJK-EPA penetration depth on the device (included by rsg_tick.cuh).
//
// Bullet runs btGjkEpa2 (B/BulletCollision/NarrowPhaseCollision/btGjkEpa2.cpp) through
// btGjkEpaPenetrationDepthSolver (btGjkEpaPenetrationDepthSolver.cpp:22-77) when its GJK pair
// detector finds the shapes overlapping beyond their margins (btGjkPairDetector.cpp:850-922).
// Citations are <file>:<line> in the RocketSim tree; B/ is libsrc/bullet3-3.24/.
//
// Everything is expressed in shape A's frame and the supports include the margins.  The polytope
// (support vertices, faces, the expansion stack) needs about 13 KB, far more than a thread can
// keep, so it lives in a work slot of a per-device pool in global memory: a thread that needs EPA
// takes a free slot with a bounded scan of atomic compare-and-swaps and gives it back afterwards.
// EPA is rare (deep box-triangle or box-sphere overlap), so the pool is small; should every slot
// be taken, the contact keeps the GJK result and the arena is flagged (WARN_EPA_SKIPPED).
#pragma once

namespace rsg {
namespace epa {

constexpr int GJK_MAX_ITER = 128;
constexpr float GJK_ACCURACY = 0.0001f, GJK_MIN_DISTANCE = 0.0001f, GJK_DUPLICATED_EPS = 0.0001f;
constexpr int EPA_MAX_VERTICES = 128, EPA_MAX_FACES = 256, EPA_MAX_ITER = 255;
constexpr float EPA_ACCURACY = 0.0001f, EPA_PLANE_EPS = 0.00001f;

struct SV {
    V3 d, w;
};
struct Face {  // EPA::sFace with indices instead of pointers
    V3 n;
    float d;
    uint8_t c[3];  // support vertices
    uint8_t e[3];  // neighbour edges
    uint8_t pass, pad;
    int16_t f[3];  // neighbour faces
    int16_t l[2];  // list links (-1: none)
};
struct Frame {  // one level of EPA::expand's recursion
    int16_t f;
    uint8_t e, stage;
};
struct Slot {
    SV sv[4 + EPA_MAX_VERTICES];  // 4 for GJK, the rest for EPA
    Face fc[EPA_MAX_FACES];
    Frame st[EPA_MAX_FACES + 1];
};

// the per-device pool (set once by the host, see rsg_kernels.cu)
__device__ uint32_t* g_epa_lock;
__device__ Slot* g_epa_slots;
__device__ int g_epa_nslots;

// btConvexShape::localGetSupportVertexNonVirtual (btConvexShape.cpp:183-193)
RSG_D V3 support_margin(const Convex& c, V3 d) {
    V3 n = d;
    if (len2(n) < SIMD_EPS * SIMD_EPS) n = V3(-1, -1, -1);
    n = normalized(n);
    return c.support_nomargin(n) + c.margin * n;
}

struct Minkowski {  // MinkowskiDiff (btGjkEpa2.cpp:80-150)
    Convex a, b;
    M3 to_b;    // direction from A's frame to B's
    Xf b_to_a;  // point from B's frame to A's
    bool margins;
    RSG_D V3 sup_a(V3 d) const { return margins ? support_margin(a, d) : a.support_nomargin(d); }
    RSG_D V3 sup_b(V3 d) const {
        V3 db = to_b * d;
        return xf_apply(b_to_a, margins ? support_margin(b, db) : b.support_nomargin(db));
    }
    RSG_D V3 sup(V3 d) const { return sup_a(d) - sup_b(-d); }
    RSG_D V3 sup(V3 d, int which) const { return which ? sup_b(d) : sup_a(d); }
};

struct Simplex {
    int c[4];
    float p[4];
    int rank;
};

RSG_D float det3(V3 a, V3 b, V3 c) {
    return (a.y * b.z * c.x + a.z * b.x * c.y - a.x * b.z * c.y - a.y * b.x * c.z + a.x * b.y * c.z - a.z * b.y * c.x);
}
RSG_D float project2(V3 a, V3 b, float* w, unsigned& m) {  // GJK::projectorigin, segment
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
RSG_D float project3(V3 a, V3 b, V3 c, float* w, unsigned& m) {  // triangle
    const int imd3[] = {1, 2, 0};
    const V3 vt[] = {a, b, c};
    const V3 dl[] = {a - b, b - c, c - a};
    const V3 n = cross(dl[0], dl[1]);
    const float l = len2(n);
    if (l > 0.f) {
        float mindist = -1;
        float subw[2] = {0.f, 0.f};
        unsigned subm = 0;
        for (int i = 0; i < 3; ++i) {
            if (dot(vt[i], cross(dl[i], n)) > 0) {
                const int j = imd3[i];
                const float subd = project2(vt[i], vt[j], subw, subm);
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
            const float s = sqrtf(l);
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
RSG_D float project4(V3 a, V3 b, V3 c, V3 d, float* w, unsigned& m) {  // tetrahedron
    const int imd3[] = {1, 2, 0};
    const V3 vt[] = {a, b, c, d};
    const V3 dl[] = {a - d, b - d, c - d};
    const float vl = det3(dl[0], dl[1], dl[2]);
    const bool ng = (vl * dot(a, cross(b - c, a - b))) <= 0;
    if (ng && (fabsf(vl) > 0.f)) {
        float mindist = -1;
        float subw[3] = {0.f, 0.f, 0.f};
        unsigned subm = 0;
        for (int i = 0; i < 3; ++i) {
            const int j = imd3[i];
            const float s = vl * dot(d, cross(dl[i], dl[j]));
            if (s > 0) {
                const float subd = project3(vt[i], vt[j], d, subw, subm);
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
            w[0] = det3(c, b, d) / vl;
            w[1] = det3(a, c, d) / vl;
            w[2] = det3(b, a, d) / vl;
            w[3] = 1 - (w[0] + w[1] + w[2]);
        }
        return mindist;
    }
    return -1;
}

// GJK of btGjkEpa2 (btGjkEpa2.cpp:155-581) over the slot's support vertices
struct Gjk {
    const Minkowski* shape;
    SV* sv;
    int freel[4], nfree;
    Simplex sims[2];
    int cur;
    V3 ray;
    int status;  // 0 valid, 1 inside, 2 failed

    RSG_D void getsupport(V3 d, SV& s) const {
        s.d = d / len(d);
        s.w = shape->sup(s.d);
    }
    RSG_D void remove_vertex(Simplex& sx) { freel[nfree++] = sx.c[--sx.rank]; }
    RSG_D void append_vertex(Simplex& sx, V3 v) {
        sx.p[sx.rank] = 0;
        sx.c[sx.rank] = freel[--nfree];
        getsupport(v, sv[sx.c[sx.rank++]]);
    }
    RSG_D int evaluate(V3 guess) {  // GJK::Evaluate (btGjkEpa2.cpp:196-324)
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
            if (cs.rank == 2) sqdist = project2(sv[cs.c[0]].w, sv[cs.c[1]].w, weights, mask);
            else if (cs.rank == 3) sqdist = project3(sv[cs.c[0]].w, sv[cs.c[1]].w, sv[cs.c[2]].w, weights, mask);
            else if (cs.rank == 4)
                sqdist = project4(sv[cs.c[0]].w, sv[cs.c[1]].w, sv[cs.c[2]].w, sv[cs.c[3]].w, weights, mask);
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
        return status;
    }
    RSG_D Simplex& simplex() { return sims[cur]; }
    // GJK::EncloseOrigin (btGjkEpa2.cpp:325-389), its recursion unrolled by simplex rank
    RSG_D bool enclose4() {
        Simplex& s = simplex();
        return fabsf(det3(sv[s.c[0]].w - sv[s.c[3]].w, sv[s.c[1]].w - sv[s.c[3]].w, sv[s.c[2]].w - sv[s.c[3]].w)) > 0;
    }
    RSG_D bool enclose3() {
        Simplex& s = simplex();
        const V3 n = cross(sv[s.c[1]].w - sv[s.c[0]].w, sv[s.c[2]].w - sv[s.c[0]].w);
        if (len2(n) > 0) {
            append_vertex(s, n);
            if (enclose4()) return true;
            remove_vertex(s);
            append_vertex(s, -n);
            if (enclose4()) return true;
            remove_vertex(s);
        }
        return false;
    }
    RSG_D bool enclose2() {
        Simplex& s = simplex();
        const V3 d = sv[s.c[1]].w - sv[s.c[0]].w;
        for (int i = 0; i < 3; ++i) {
            V3 axis(0, 0, 0);
            axis[i] = 1;
            const V3 p = cross(d, axis);
            if (len2(p) > 0) {
                append_vertex(s, p);
                if (enclose3()) return true;
                remove_vertex(s);
                append_vertex(s, -p);
                if (enclose3()) return true;
                remove_vertex(s);
            }
        }
        return false;
    }
    RSG_D bool enclose1() {
        Simplex& s = simplex();
        for (int i = 0; i < 3; ++i) {
            V3 axis(0, 0, 0);
            axis[i] = 1;
            append_vertex(s, axis);
            if (enclose2()) return true;
            remove_vertex(s);
            append_vertex(s, -axis);
            if (enclose2()) return true;
            remove_vertex(s);
        }
        return false;
    }
    RSG_D bool enclose_origin() {
        switch (simplex().rank) {
            case 1: return enclose1();
            case 2: return enclose2();
            case 3: return enclose3();
            case 4: return enclose4();
        }
        return false;
    }
};

struct List {
    int root, count;
};

// EPA (btGjkEpa2.cpp:583-950) over the slot's faces
struct Epa {
    Face* fc;
    Frame* st;
    List hull, stock;
    int nextsv;
    int status;  // eStatus: 0 valid ... 8 fallback, 9 failed
    V3 normal;
    float depth;
    Simplex result;

    RSG_D void bind(int fa, int ea, int fb, int eb) {
        fc[fa].e[ea] = (uint8_t)eb;
        fc[fa].f[ea] = (int16_t)fb;
        fc[fb].e[eb] = (uint8_t)ea;
        fc[fb].f[eb] = (int16_t)fa;
    }
    RSG_D void append(List& list, int face) {
        fc[face].l[0] = -1;
        fc[face].l[1] = (int16_t)list.root;
        if (list.root >= 0) fc[list.root].l[0] = (int16_t)face;
        list.root = face;
        ++list.count;
    }
    RSG_D void remove(List& list, int face) {
        if (fc[face].l[1] >= 0) fc[fc[face].l[1]].l[0] = fc[face].l[0];
        if (fc[face].l[0] >= 0) fc[fc[face].l[0]].l[1] = fc[face].l[1];
        if (face == list.root) list.root = fc[face].l[1];
        --list.count;
    }
    RSG_D void init() {
        status = 9;
        normal = V3(0, 0, 0);
        depth = 0;
        nextsv = 0;
        hull.root = stock.root = -1;
        hull.count = stock.count = 0;
        for (int i = 0; i < EPA_MAX_FACES; ++i) append(stock, EPA_MAX_FACES - i - 1);
    }
    RSG_D bool edge_dist(const Gjk& g, int face, int a, int b, float& dist) const {
        const V3 aw = g.sv[a].w, bw = g.sv[b].w;
        const V3 ba = bw - aw;
        const V3 n_ab = cross(ba, fc[face].n);
        if (dot(aw, n_ab) < 0) {
            const float ba_l2 = len2(ba);
            const float a_dot_ba = dot(aw, ba);
            const float b_dot_ba = dot(bw, ba);
            if (a_dot_ba > 0) dist = len(aw);
            else if (b_dot_ba < 0) dist = len(bw);
            else {
                const float a_dot_b = dot(aw, bw);
                float v = (len2(aw) * len2(bw) - a_dot_b * a_dot_b) / ba_l2;
                dist = sqrtf(v > 0.f ? v : 0.f);
            }
            return true;
        }
        return false;
    }
    RSG_D int newface(const Gjk& g, int a, int b, int c, bool forced) {
        if (stock.root >= 0) {
            const int face = stock.root;
            remove(stock, face);
            append(hull, face);
            Face& F = fc[face];
            F.pass = 0;
            F.c[0] = (uint8_t)a;
            F.c[1] = (uint8_t)b;
            F.c[2] = (uint8_t)c;
            F.n = cross(g.sv[b].w - g.sv[a].w, g.sv[c].w - g.sv[a].w);
            const float l = len(F.n);
            if (l > EPA_ACCURACY) {
                float d = 0;
                if (!(edge_dist(g, face, a, b, d) || edge_dist(g, face, b, c, d) || edge_dist(g, face, c, a, d)))
                    d = dot(g.sv[a].w, F.n) / l;
                F.d = d;
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
    RSG_D int findbest() const {
        int minf = hull.root;
        float mind = fc[minf].d * fc[minf].d;
        for (int f = fc[minf].l[1]; f >= 0; f = fc[f].l[1]) {
            const float sqd = fc[f].d * fc[f].d;
            if (sqd < mind) { minf = f; mind = sqd; }
        }
        return minf;
    }
    // EPA::expand (btGjkEpa2.cpp:912-948), its recursion on an explicit stack in the slot
    RSG_D bool expand(const Gjk& g, int pass, int w, int f0, int e0, int& hcf, int& hff, int& hnf) {
        const int i1m3[] = {1, 2, 0};
        const int i2m3[] = {2, 0, 1};
        int sp = 0;
        st[sp].f = (int16_t)f0; st[sp].e = (uint8_t)e0; st[sp].stage = 0; sp++;
        bool ret = false;
        while (sp > 0) {
            Frame& fr = st[sp - 1];
            Face& F = fc[fr.f];
            if (fr.stage == 0) {
                if (F.pass == pass) { ret = false; sp--; continue; }
                const int e1 = i1m3[fr.e];
                if ((dot(F.n, g.sv[w].w) - F.d) < -EPA_PLANE_EPS) {
                    const int nf = newface(g, F.c[e1], F.c[fr.e], w, false);
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
                st[sp].f = F.f[e1]; st[sp].e = F.e[e1]; st[sp].stage = 0; sp++;
                continue;
            }
            if (fr.stage == 1) {
                if (!ret) { sp--; continue; }
                fr.stage = 2;
                const int e2 = i2m3[fr.e];
                st[sp].f = F.f[e2]; st[sp].e = F.e[e2]; st[sp].stage = 0; sp++;
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
    RSG_D int evaluate(Gjk& g, V3 guess) {
        Simplex& sx = g.simplex();
        if ((sx.rank > 1) && g.enclose_origin()) {
            while (hull.root >= 0) {
                const int f = hull.root;
                remove(hull, f);
                append(stock, f);
            }
            status = 0;
            nextsv = 0;
            if (det3(g.sv[sx.c[0]].w - g.sv[sx.c[3]].w, g.sv[sx.c[1]].w - g.sv[sx.c[3]].w,
                     g.sv[sx.c[2]].w - g.sv[sx.c[3]].w) < 0) {
                int tc = sx.c[0]; sx.c[0] = sx.c[1]; sx.c[1] = tc;
                float tp = sx.p[0]; sx.p[0] = sx.p[1]; sx.p[1] = tp;
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
RSG_D void setup(Minkowski& m, const Convex& a, const Xf& ta, const Convex& b, const Xf& tb, bool margins) {
    m.a = a;
    m.b = b;
    m.to_b = transpose_times(tb.b, ta.b);
    Xf r;  // btTransform::inverseTimes
    r.b = transpose_times(ta.b, tb.b);
    r.o = (tb.o - ta.o) * ta.b;
    m.b_to_a = r;
    m.margins = margins;
}

// btGjkEpaPenetrationDepthSolver::calcPenDepth (btGjkEpaPenetrationDepthSolver.cpp:22-77) with
// btGjkEpaSolver2::Penetration and ::Distance (btGjkEpa2.cpp:979-1052) inlined
RSG_DN bool calc_pen_depth(const Convex& a, const Xf& ta, const Convex& b, const Xf& tb, Slot* slot, V3& v, V3& wa,
                           V3& wb) {
    const V3 guesses[9] = {safe_normalized(tb.o - ta.o), safe_normalized(ta.o - tb.o), V3(0, 0, 1), V3(0, 1, 0),
                           V3(1, 0, 0), V3(1, 1, 0), V3(1, 1, 1), V3(0, 1, 1), V3(1, 0, 1)};
    Minkowski mk;
    Gjk g;
    g.shape = &mk;
    g.sv = slot->sv;
    for (int gi = 0; gi < 9; gi++) {
        const V3 guess = guesses[gi];
        // Penetration: GJK with margins from -guess; EPA when the origin is inside
        setup(mk, a, ta, b, tb, true);
        if (g.evaluate(-guess) == 1) {
            Epa e;
            e.fc = slot->fc;
            e.st = slot->st;
            e.init();
            if (e.evaluate(g, -guess) != 9) {
                V3 w0(0, 0, 0);
                for (int i = 0; i < e.result.rank; ++i) w0 += mk.sup(g.sv[e.result.c[i]].d, 0) * e.result.p[i];
                wa = xf_apply(ta, w0);
                wb = xf_apply(ta, w0 - e.normal * e.depth);
                v = -e.normal;
                return true;
            }
        }
        // Distance: GJK without margins from guess
        setup(mk, a, ta, b, tb, false);
        if (g.evaluate(guess) == 0) {
            Simplex& s = g.simplex();
            V3 w0(0, 0, 0), w1(0, 0, 0);
            for (int i = 0; i < s.rank; ++i) {
                const float p = s.p[i];
                w0 += mk.sup(g.sv[s.c[i]].d, 0) * p;
                w1 += mk.sup(-g.sv[s.c[i]].d, 1) * p;
            }
            wa = xf_apply(ta, w0);
            wb = xf_apply(ta, w1);
            V3 n = w0 - w1;
            const float dist = len(n);
            v = n / (dist > GJK_MIN_DISTANCE ? dist : 1);
            return false;
        }
    }
    wa = wb = v = V3(0, 0, 0);
    return false;
}

// A free work slot of the pool, or -1 (a bounded scan, no waiting)
RSG_D int acquire_slot() {
    const int n = g_epa_nslots;
    if (n <= 0 || !g_epa_lock) return -1;
    const int start = (int)((blockIdx.x * 131u + threadIdx.x) % (unsigned)n);
    for (int k = 0; k < n; k++) {
        const int s = (start + k) % n;
        if (atomicCAS(&g_epa_lock[s], 0u, 1u) == 0u) return s;
    }
    return -1;
}
RSG_D void release_slot(int s) {
    __threadfence();
    atomicExch(&g_epa_lock[s], 0u);
}

}  // namespace epa
}  // namespace rsg
