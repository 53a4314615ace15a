/*
 * Embree 3 stand-in for the reference-renderer build (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
 *
 * Embree is absent, so the reference's own Scene / TriangleMesh / Instance code (src/core/Scene.cpp,
 * TriangleMesh.cpp:57-63, Instance.cpp:11-34) is linked against this implementation of the 18 rtc*
 * calls it makes.  Semantics restated from Embree 3's public documentation, as the reference uses
 * them: tnear = 0 and tfar = inf on entry; a closest hit writes ray.tfar, hit.u / hit.v with
 * p = (1 - u - v) p0 + u p1 + v p2, the unnormalised geometric normal Ng = cross(p1 - p0, p2 - p0)
 * in the space of the hit geometry (object space for an instance), primID, geomID (the id inside
 * the instanced scene for an instance hit) and instID[0] (the instance's id, or
 * RTC_INVALID_GEOMETRY_ID); rtcOccluded1 sets ray.tfar = -inf when any triangle lies at t in
 * (0, tfar].  One instancing level.
 *
 * The acceleration structure and the triangle test are the ones the CPU oracle uses (binned SAH
 * over 16 bins, leaves of 4 triangles under one leaf per geometry at the top, a two-sided
 * Moller-Trumbore test, the instance ray moved into object space by the double-precision inverse
 * of the 3x4 transform), built in the same order, so both programs report the same hit for every
 * ray -- including ties -- and the per-path comparison of the two integrators isolates their own
 * arithmetic.
 */
#include <embree3/rtcore.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <memory>
#include <vector>

namespace {

const float INF = std::numeric_limits<float>::infinity();

struct V { float x = 0, y = 0, z = 0; };
inline V mk(float a, float b, float c) { V r; r.x = a; r.y = b; r.z = c; return r; }
inline V sub(const V &a, const V &b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V add(const V &a, const V &b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V scale(const V &a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline float dot(const V &a, const V &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(const V &a, const V &b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float comp(const V &a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
/* column-major 3x3 times a vector, in the order m0 x + m3 y + m6 z */
inline V mulcm(const float *m, const V &v) {
    return mk(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z, m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

struct Box {
    V lo, hi;
    float area() const { const V s = sub(hi, lo); return (s.x * s.y + s.y * s.z + s.x * s.z) * 2.f; }
    V centre() const { return add(lo, scale(sub(hi, lo), .5f)); }
};
inline Box box_of(const V &p) { Box b; b.lo = p; b.hi = p; return b; }
inline Box join(const Box &a, const Box &b) {
    Box r;
    r.lo = mk(std::min(a.lo.x, b.lo.x), std::min(a.lo.y, b.lo.y), std::min(a.lo.z, b.lo.z));
    r.hi = mk(std::max(a.hi.x, b.hi.x), std::max(a.hi.y, b.hi.y), std::max(a.hi.z, b.hi.z));
    return r;
}
inline Box join(const Box &b, const V &p) {
    Box r;
    r.lo = mk(std::min(p.x, b.lo.x), std::min(p.y, b.lo.y), std::min(p.z, b.lo.z));
    r.hi = mk(std::max(p.x, b.hi.x), std::max(p.y, b.hi.y), std::max(p.z, b.hi.z));
    return r;
}

struct Node { Box b; int left = -1, right = -1, first = 0, count = 0; };

/* Binned-SAH BVH2 over primitive boxes, depth-first with an explicit job stack. */
void build_bvh(std::vector<Node> &nodes, std::vector<uint32_t> &idx, const std::vector<Box> &pb, const std::vector<V> &pc,
               int leaf_max) {
    const size_t n = pb.size();
    idx.resize(n);
    for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    nodes.clear();
    if (n == 0) return;
    nodes.reserve(2 * n + 1);
    struct Job { int node, first, count; };
    std::vector<Job> jobs;
    nodes.push_back(Node());
    jobs.push_back({0, 0, (int)n});
    const int NB = 16;
    while (!jobs.empty()) {
        const Job j = jobs.back();
        jobs.pop_back();
        Box b = pb[idx[j.first]], cb = box_of(pc[idx[j.first]]);
        for (int i = j.first; i < j.first + j.count; ++i) { b = join(b, pb[idx[i]]); cb = join(cb, pc[idx[i]]); }
        nodes[j.node].b = b;
        if (j.count <= leaf_max) { nodes[j.node].first = j.first; nodes[j.node].count = j.count; continue; }
        int best_axis = -1, best_split = -1;
        float best_cost = INF;
        for (int ax = 0; ax < 3; ++ax) {
            const float lo = comp(cb.lo, ax), hi = comp(cb.hi, ax);
            if (!(hi > lo)) continue;
            Box bins[NB];
            int cnt[NB] = {0};
            bool used[NB] = {false};
            for (int i = j.first; i < j.first + j.count; ++i) {
                int k = (int)((comp(pc[idx[i]], ax) - lo) / (hi - lo) * NB);
                k = k >= NB ? NB - 1 : (k < 0 ? 0 : k);
                bins[k] = used[k] ? join(bins[k], pb[idx[i]]) : pb[idx[i]];
                used[k] = true;
                cnt[k]++;
            }
            float right_area[NB];
            int right_cnt[NB];
            {
                Box acc;
                bool any = false;
                int c = 0;
                for (int k = NB - 1; k > 0; --k) {
                    if (used[k]) { acc = any ? join(acc, bins[k]) : bins[k]; any = true; }
                    c += cnt[k];
                    right_area[k] = any ? acc.area() : 0.f;
                    right_cnt[k] = c;
                }
            }
            Box acc;
            bool any = false;
            int c = 0;
            for (int k = 0; k < NB - 1; ++k) {
                if (used[k]) { acc = any ? join(acc, bins[k]) : bins[k]; any = true; }
                c += cnt[k];
                if (c == 0 || right_cnt[k + 1] == 0) continue;
                const float cost = acc.area() * c + right_area[k + 1] * right_cnt[k + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_split = k; }
            }
        }
        int mid;
        if (best_axis < 0) {
            mid = j.first + j.count / 2;
        } else {
            const float lo = comp(cb.lo, best_axis), hi = comp(cb.hi, best_axis);
            uint32_t *beg = &idx[j.first], *end = beg + j.count;
            uint32_t *m = std::partition(beg, end, [&](uint32_t p) {
                int k = (int)((comp(pc[p], best_axis) - lo) / (hi - lo) * NB);
                k = k >= NB ? NB - 1 : (k < 0 ? 0 : k);
                return k <= best_split;
            });
            mid = (int)(m - &idx[0]);
            if (mid == j.first || mid == j.first + j.count) mid = j.first + j.count / 2;
        }
        const int l = (int)nodes.size();
        nodes.push_back(Node());
        const int r = (int)nodes.size();
        nodes.push_back(Node());
        nodes[j.node].left = l;
        nodes[j.node].right = r;
        jobs.push_back({l, j.first, mid - j.first});
        jobs.push_back({r, mid, j.first + j.count - mid});
    }
}

/* two-sided Moller-Trumbore; accepts 0 < t < tmax */
inline bool hit_tri(const V &o, const V &d, const V &p0, const V &p1, const V &p2, float tmax, float *t, float *u, float *v) {
    const V e1 = sub(p1, p0), e2 = sub(p2, p0);
    const V pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0) return false;
    const float inv = 1.f / det;
    const V tv = sub(o, p0);
    const float uu = dot(tv, pv) * inv;
    if (uu < 0 || uu > 1) return false;
    const V qv = cross(tv, e1);
    const float vv = dot(d, qv) * inv;
    if (vv < 0 || uu + vv > 1) return false;
    const float tt = dot(e2, qv) * inv;
    if (!(tt > 0) || !(tt < tmax)) return false;
    *t = tt; *u = uu; *v = vv;
    return true;
}
inline bool hit_box(const Box &b, const V &o, const V &inv, float tmax) {
    float t0 = 0, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        float ta = (comp(b.lo, a) - comp(o, a)) * comp(inv, a), tb = (comp(b.hi, a) - comp(o, a)) * comp(inv, a);
        if (ta > tb) std::swap(ta, tb);
        if (!(ta <= tb)) { ta = -INF; tb = INF; }   /* 0 * inf on a slab plane: inside */
        t0 = ta > t0 ? ta : t0;
        t1 = tb < t1 ? tb : t1;
        if (t0 > t1) return false;
    }
    return true;
}

void inverse3(const float *m, float *inv) {   /* column-major m, inverse in double, stored column-major */
    const double a = m[0], b = m[3], c = m[6], dd = m[1], e = m[4], f = m[7], g = m[2], h = m[5], i = m[8];
    const double A = e * i - f * h, B = -(dd * i - f * g), C = dd * h - e * g;
    const double det = a * A + b * B + c * C;
    const double id = 1.0 / det;
    const double r[9] = {A * id, -(b * i - c * h) * id, (b * f - c * e) * id,
                         B * id, (a * i - c * g) * id, -(a * f - c * dd) * id,
                         C * id, -(a * h - b * g) * id, (a * e - b * dd) * id};
    inv[0] = (float)r[0]; inv[3] = (float)r[1]; inv[6] = (float)r[2];
    inv[1] = (float)r[3]; inv[4] = (float)r[4]; inv[7] = (float)r[5];
    inv[2] = (float)r[6]; inv[5] = (float)r[7]; inv[8] = (float)r[8];
}

}  // namespace

struct RTCDeviceTy { int unused = 0; };
struct RTCSceneTy;
struct RTCGeometryTy {
    RTCGeometryType type;
    /* triangles: shared buffers (TriangleMesh::Commit, TriangleMesh.cpp:57-63) */
    const unsigned char *vtx = nullptr, *idx = nullptr;
    size_t vtx_stride = 0, idx_stride = 0, n_vtx = 0, n_tri = 0;
    std::vector<Node> nodes;
    std::vector<uint32_t> tri_order;
    /* instances */
    RTCSceneTy *inst = nullptr;
    float xfm[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    float minv[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    bool identity = true;
    V vert(uint32_t i) const { const float *p = reinterpret_cast<const float *>(vtx + i * vtx_stride); return mk(p[0], p[1], p[2]); }
    void tri(uint32_t t, uint32_t out[3]) const {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(idx + t * idx_stride);
        out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
    }
};
struct RTCSceneTy {
    std::vector<RTCGeometry> geoms;   /* by geometry id; null = free */
    std::vector<Node> top;
    std::vector<uint32_t> top_order;
    std::vector<unsigned> top_ids;    /* leaf slot -> geometry id */
    Box bounds;
    bool has_bounds = false;
};

namespace {

/* world bounds of a geometry: its vertices, moved by the instance transform (x' = M x + t) */
Box geom_bounds(const RTCGeometryTy *g) {
    if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) {
        Box b = box_of(g->vert(0));
        for (size_t i = 1; i < g->n_vtx; ++i) b = join(b, g->vert((uint32_t)i));
        return b;
    }
    const RTCGeometryTy *m = nullptr;
    for (RTCGeometry q : g->inst->geoms) if (q) { m = q; break; }
    Box b;
    bool first = true;
    const V t = mk(g->xfm[9], g->xfm[10], g->xfm[11]);
    for (size_t i = 0; m && i < m->n_vtx; ++i) {
        const V v = m->vert((uint32_t)i);
        const V w = g->identity ? v : add(mulcm(g->xfm, v), t);
        b = first ? box_of(w) : join(b, w);
        first = false;
    }
    return b;
}

void build_mesh(RTCGeometryTy *g) {
    std::vector<Box> pb(g->n_tri);
    std::vector<V> pc(g->n_tri);
    for (size_t i = 0; i < g->n_tri; ++i) {
        uint32_t t[3];
        g->tri((uint32_t)i, t);
        Box b = box_of(g->vert(t[0]));
        b = join(b, g->vert(t[1]));
        b = join(b, g->vert(t[2]));
        pb[i] = b;
        pc[i] = b.centre();
    }
    build_bvh(g->nodes, g->tri_order, pb, pc, 4);
}

struct Best { float t, u, v; unsigned prim, geom, inst; V ng; };

/* closest (any = false) or any hit of one triangle geometry, ray in its space */
bool trace_mesh(const RTCGeometryTy *g, const V &o, const V &d, float &tmax, bool any, Best *best) {
    if (g->nodes.empty()) return false;
    const V inv = mk(1 / d.x, 1 / d.y, 1 / d.z);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    bool found = false;
    while (sp) {
        const Node &nd = g->nodes[stack[--sp]];
        if (!hit_box(nd.b, o, inv, tmax)) continue;
        if (nd.left < 0) {
            for (int q = nd.first; q < nd.first + nd.count; ++q) {
                const uint32_t ti = g->tri_order[q];
                uint32_t t[3];
                g->tri(ti, t);
                const V p0 = g->vert(t[0]), p1 = g->vert(t[1]), p2 = g->vert(t[2]);
                float tt, uu, vv;
                if (hit_tri(o, d, p0, p1, p2, tmax, &tt, &uu, &vv)) {
                    if (any) return true;
                    tmax = tt;
                    best->t = tt; best->u = uu; best->v = vv; best->prim = ti;
                    best->ng = cross(sub(p1, p0), sub(p2, p0));
                    found = true;
                }
            }
        } else {
            stack[sp++] = nd.right;
            stack[sp++] = nd.left;
        }
    }
    return found;
}

/* top level: every geometry of the scene, instances entered with the ray in object space */
bool trace_scene(const RTCSceneTy *s, const V &o, const V &d, float tmax, bool any, Best *best) {
    if (s->top.empty()) return false;
    const V inv = mk(1 / d.x, 1 / d.y, 1 / d.z);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    bool found = false;
    while (sp) {
        const Node &nd = s->top[stack[--sp]];
        if (!hit_box(nd.b, o, inv, tmax)) continue;
        if (nd.left < 0) {
            for (int k = nd.first; k < nd.first + nd.count; ++k) {
                const unsigned id = s->top_ids[s->top_order[k]];
                const RTCGeometryTy *g = s->geoms[id];
                if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) {
                    if (trace_mesh(g, o, d, tmax, any, best)) {
                        if (any) return true;
                        best->geom = id; best->inst = RTC_INVALID_GEOMETRY_ID;
                        found = true;
                    }
                } else {
                    V oo = o, dd = d;
                    if (!g->identity) {
                        oo = mulcm(g->minv, sub(o, mk(g->xfm[9], g->xfm[10], g->xfm[11])));
                        dd = mulcm(g->minv, d);
                    }
                    for (size_t j = 0; j < g->inst->geoms.size(); ++j) {
                        const RTCGeometryTy *m = g->inst->geoms[j];
                        if (!m || m->type != RTC_GEOMETRY_TYPE_TRIANGLE) continue;
                        if (trace_mesh(m, oo, dd, tmax, any, best)) {
                            if (any) return true;
                            best->geom = (unsigned)j; best->inst = id;
                            found = true;
                        }
                    }
                }
            }
        } else {
            stack[sp++] = nd.right;
            stack[sp++] = nd.left;
        }
    }
    return found;
}

}  // namespace

RTCDevice rtcNewDevice(const char *) { return new RTCDeviceTy(); }
RTCScene rtcNewScene(RTCDevice) { return new RTCSceneTy(); }
void rtcSetSceneFlags(RTCScene, RTCSceneFlags) {}
void rtcSetSceneBuildQuality(RTCScene, RTCBuildQuality) {}

void rtcCommitScene(RTCScene s) {
    std::vector<Box> pb;
    std::vector<V> pc;
    s->top_ids.clear();
    s->has_bounds = false;
    for (size_t id = 0; id < s->geoms.size(); ++id) {
        RTCGeometryTy *g = s->geoms[id];
        if (!g) continue;
        if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE && g->nodes.empty() && g->n_tri) build_mesh(g);
        const Box b = geom_bounds(g);
        pb.push_back(b);
        pc.push_back(b.centre());
        s->top_ids.push_back((unsigned)id);
        s->bounds = s->has_bounds ? join(s->bounds, b) : b;
        s->has_bounds = true;
    }
    build_bvh(s->top, s->top_order, pb, pc, 1);
}

void rtcGetSceneBounds(RTCScene s, RTCBounds *b) {
    const Box x = s->has_bounds ? s->bounds : Box();
    b->lower_x = x.lo.x; b->lower_y = x.lo.y; b->lower_z = x.lo.z; b->align0 = 0;
    b->upper_x = x.hi.x; b->upper_y = x.hi.y; b->upper_z = x.hi.z; b->align1 = 0;
}

void rtcIntersect1(RTCScene s, RTCIntersectContext *, RTCRayHit *rh) {
    RTCRay &r = rh->ray;
    Best best;
    best.prim = best.geom = best.inst = RTC_INVALID_GEOMETRY_ID;
    if (trace_scene(s, mk(r.org_x, r.org_y, r.org_z), mk(r.dir_x, r.dir_y, r.dir_z), r.tfar, false, &best)) {
        r.tfar = best.t;
        rh->hit.u = best.u; rh->hit.v = best.v;
        rh->hit.Ng_x = best.ng.x; rh->hit.Ng_y = best.ng.y; rh->hit.Ng_z = best.ng.z;
        rh->hit.primID = best.prim;
        rh->hit.geomID = best.geom;
        rh->hit.instID[0] = best.inst;
    } else {
        rh->hit.geomID = RTC_INVALID_GEOMETRY_ID;
        rh->hit.primID = RTC_INVALID_GEOMETRY_ID;
        rh->hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
    }
}

void rtcOccluded1(RTCScene s, RTCIntersectContext *, RTCRay *r) {
    Best best;
    /* t in (0, tfar]: the triangle test is strict, so widen its bound by one ulp */
    const float lim = std::nextafter(r->tfar, INF);
    if (trace_scene(s, mk(r->org_x, r->org_y, r->org_z), mk(r->dir_x, r->dir_y, r->dir_z), lim, true, &best)) r->tfar = -INF;
}

unsigned rtcAttachGeometry(RTCScene s, RTCGeometry g) {
    for (size_t i = 0; i < s->geoms.size(); ++i)
        if (!s->geoms[i]) { s->geoms[i] = g; return (unsigned)i; }
    s->geoms.push_back(g);
    return (unsigned)(s->geoms.size() - 1);
}
void rtcAttachGeometryByID(RTCScene s, RTCGeometry g, unsigned id) {
    if (s->geoms.size() <= id) s->geoms.resize(id + 1, nullptr);
    s->geoms[id] = g;
}
void rtcDetachGeometry(RTCScene s, unsigned id) {
    if (id < s->geoms.size()) s->geoms[id] = nullptr;
}
RTCGeometry rtcNewGeometry(RTCDevice, RTCGeometryType t) {
    RTCGeometryTy *g = new RTCGeometryTy();
    g->type = t;
    return g;
}
void rtcSetSharedGeometryBuffer(RTCGeometry g, RTCBufferType type, unsigned, RTCFormat, const void *ptr, size_t offset,
                                size_t stride, size_t count) {
    const unsigned char *p = static_cast<const unsigned char *>(ptr) + offset;
    if (type == RTC_BUFFER_TYPE_VERTEX) { g->vtx = p; g->vtx_stride = stride; g->n_vtx = count; }
    else { g->idx = p; g->idx_stride = stride; g->n_tri = count; }
    g->nodes.clear();
}
void rtcRetainGeometry(RTCGeometry) {}
void rtcCommitGeometry(RTCGeometry g) {
    if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) { g->nodes.clear(); if (g->n_tri) build_mesh(g); }
}
void rtcSetGeometryInstancedScene(RTCGeometry g, RTCScene s) { g->inst = s; }
void rtcSetGeometryTransform(RTCGeometry g, unsigned, RTCFormat, const void *xfm) {
    const float *m = static_cast<const float *>(xfm);
    static const float id[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    g->identity = true;
    for (int k = 0; k < 12; ++k) {
        g->xfm[k] = m[k];
        if (m[k] != id[k]) g->identity = false;
    }
    inverse3(g->xfm, g->minv);
}
void rtcCollide(RTCScene, RTCScene, RTCCollideFunc, void *) {}
