/*
 * Scene compilation on the host: BVH2 build and shader-graph bytecode compiler.
 *
 * BVH: centroid-binned SAH (16 bins), leaves of at most `max_leaf` primitives, object-median
 * fallback below depth 40 so every traversal stack stays under 64 entries.
 *
 * Shader graphs: the reference evaluates a node graph by pulling sockets through delegates on every
 * query, re-evaluating shared subgraphs each time (src/shading/graph/ShaderGraph.h:82-251).  Every
 * node is a pure function of the shading event, so the compiler walks the DAG once from the root,
 * memoises each (node, output) -- common-subexpression elimination -- and emits one instruction per
 * node plus the explicit type conversions that Socket::GetAs<T> performs implicitly.  A linear-scan
 * allocator maps the SSA values onto LGPU_MAX_REGS float4 registers.
 */
#include <algorithm>
#include <deque>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <thread>

#include "lgpu_build.h"
#include "lgpu_device.cuh"

namespace lg {

/* ------------------------------------------------------------------ BVH */
namespace {
struct BuildJob { int node, first, count, depth; };

inline float area(const Aabb &b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.f * (dx * dy + dy * dz + dz * dx);
}
inline void grow(Aabb &a, const Aabb &b) {
    for (int k = 0; k < 3; ++k) { a.lo[k] = std::min(a.lo[k], b.lo[k]); a.hi[k] = std::max(a.hi[k], b.hi[k]); }
}
inline Aabb empty_box() {
    Aabb b;
    for (int k = 0; k < 3; ++k) { b.lo[k] = INFINITY; b.hi[k] = -INFINITY; }
    return b;
}
}  // namespace

void build_bvh(const std::vector<Aabb> &boxes, int max_leaf, int node_base, int prim_base, BvhOut &out) {
    const int n = (int)boxes.size();
    out.nodes.clear();
    out.order.resize(n);
    out.max_depth = 0;
    for (int i = 0; i < n; ++i) out.order[i] = (uint32_t)i;
    if (n == 0) {
        DNode e;
        e.xs = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
        e.ys = e.xs; e.zs = e.xs;
        e.ch = make_int4(0, 0, 0, 0);
        out.nodes.push_back(e);
        out.root_ref = (node_base << 4);
        return;
    }
    std::vector<float> cen(3 * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cen[3 * (size_t)i + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
    if (n <= max_leaf) {   /* single leaf root */
        out.root_ref = ((prim_base) << 4) | n;
        DNode e;
        e.xs = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
        e.ys = e.xs; e.zs = e.xs;
        e.ch = make_int4(0, 0, 0, 0);
        out.nodes.push_back(e);   /* unused placeholder keeps node numbering simple */
        return;
    }
    uint32_t *idx = out.order.data();
    const int NB = 16;
    out.nodes.reserve(2 * (size_t)n / std::max(1, max_leaf) + 16);
    /* a job describes a range that must become child `slot` of parent `node` */
    struct Job { int parent, slot, first, count, depth; };
    std::vector<Job> stack;
    out.nodes.push_back(DNode());
    /* root: split directly */
    stack.push_back({-1, 0, 0, n, 0});
    while (!stack.empty()) {
        const Job j = stack.back();
        stack.pop_back();
        Aabb box = empty_box(), cb = empty_box();
        for (int i = j.first; i < j.first + j.count; ++i) {
            grow(box, boxes[idx[i]]);
            const float *c = &cen[3 * (size_t)idx[i]];
            for (int k = 0; k < 3; ++k) { cb.lo[k] = std::min(cb.lo[k], c[k]); cb.hi[k] = std::max(cb.hi[k], c[k]); }
        }
        out.max_depth = std::max(out.max_depth, j.depth);
        int ref;
        int nodeIdx = -1;
        if (j.count <= max_leaf) {
            ref = ((prim_base + j.first) << 4) | j.count;
        } else {
            nodeIdx = (j.parent < 0) ? 0 : (int)out.nodes.size();
            if (j.parent >= 0) out.nodes.push_back(DNode());
            ref = (node_base + nodeIdx) << 4;
        }
        if (j.parent >= 0) {
            DNode &p = out.nodes[j.parent];
            if (j.slot == 0) {
                p.xs.x = box.lo[0]; p.xs.y = box.hi[0]; p.ys.x = box.lo[1]; p.ys.y = box.hi[1]; p.zs.x = box.lo[2]; p.zs.y = box.hi[2];
                p.ch.x = ref;
            } else {
                p.xs.z = box.lo[0]; p.xs.w = box.hi[0]; p.ys.z = box.lo[1]; p.ys.w = box.hi[1]; p.zs.z = box.lo[2]; p.zs.w = box.hi[2];
                p.ch.y = ref;
            }
        } else {
            out.root_ref = ref;
        }
        if (nodeIdx < 0) continue;
        /* choose a split */
        int bestAxis = -1, bestSplit = -1;
        float bestCost = INFINITY;
        if (j.depth < 40) {
            for (int ax = 0; ax < 3; ++ax) {
                const float lo = cb.lo[ax], hi = cb.hi[ax];
                if (!(hi > lo)) continue;
                const float scale = (float)NB / (hi - lo);
                Aabb bb[NB];
                int cnt[NB];
                for (int b = 0; b < NB; ++b) { bb[b] = empty_box(); cnt[b] = 0; }
                for (int i = j.first; i < j.first + j.count; ++i) {
                    int b = (int)((cen[3 * (size_t)idx[i] + ax] - lo) * scale);
                    b = std::min(std::max(b, 0), NB - 1);
                    grow(bb[b], boxes[idx[i]]);
                    cnt[b]++;
                }
                float rA[NB];
                int rC[NB];
                Aabb acc = empty_box();
                int c = 0;
                for (int b = NB - 1; b > 0; --b) { grow(acc, bb[b]); c += cnt[b]; rA[b] = area(acc); rC[b] = c; }
                acc = empty_box();
                c = 0;
                for (int b = 0; b < NB - 1; ++b) {
                    grow(acc, bb[b]);
                    c += cnt[b];
                    if (c == 0 || rC[b + 1] == 0) continue;
                    const float cost = area(acc) * (float)c + rA[b + 1] * (float)rC[b + 1];
                    if (cost < bestCost) { bestCost = cost; bestAxis = ax; bestSplit = b; }
                }
            }
        }
        int mid;
        if (bestAxis < 0) {
            /* object median on the widest centroid axis */
            int ax = 0;
            for (int k = 1; k < 3; ++k) if (cb.hi[k] - cb.lo[k] > cb.hi[ax] - cb.lo[ax]) ax = k;
            mid = j.first + j.count / 2;
            std::nth_element(idx + j.first, idx + mid, idx + j.first + j.count, [&](uint32_t a, uint32_t b) {
                return cen[3 * (size_t)a + ax] < cen[3 * (size_t)b + ax];
            });
        } else {
            const float lo = cb.lo[bestAxis], hi = cb.hi[bestAxis];
            const float scale = (float)NB / (hi - lo);
            uint32_t *m = std::partition(idx + j.first, idx + j.first + j.count, [&](uint32_t p) {
                int b = (int)((cen[3 * (size_t)p + bestAxis] - lo) * scale);
                b = std::min(std::max(b, 0), NB - 1);
                return b <= bestSplit;
            });
            mid = (int)(m - idx);
            if (mid == j.first || mid == j.first + j.count) mid = j.first + j.count / 2;
        }
        stack.push_back({nodeIdx, 1, mid, j.first + j.count - mid, j.depth + 1});
        stack.push_back({nodeIdx, 0, j.first, mid - j.first, j.depth + 1});
    }
}

/* ------------------------------------------------------------------ 8-wide collapse */
namespace {

struct WideCand {
    Aabb box;
    int ref;
};

/* decoded plane p + q * s (q * s exact): the expression the traversal evaluates */
inline float wide_plane(float p, int q, float s) {
    const float qs = (float)q * s;
    return p + qs;
}
inline float wide_scale(int e) {   /* 2^(e - 127), e in 1..254 */
    uint32_t b = (uint32_t)e << 23;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

/* Quantisation frame of a node box and the outward-rounded 8-bit planes of its children. */
void quantise(DWide &w, const Aabb &node, const std::vector<WideCand> &ch) {
    const float p[3] = {node.lo[0], node.lo[1], node.lo[2]};
    w.px = p[0]; w.py = p[1]; w.pz = p[2];
    int e[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = node.hi[a] - node.lo[a];
        int ee = 1;
        if (ext > 0.f && std::isfinite(ext)) {
            int x2;
            std::frexp(ext / 255.f, &x2);   /* ext / 255 < 2^x2 */
            ee = std::min(std::max(x2 + 127, 1), 254);
        }
        while (ee < 254 && wide_plane(p[a], 255, wide_scale(ee)) < node.hi[a]) ++ee;
        e[a] = ee;
    }
    w.ex = (uint8_t)e[0]; w.ey = (uint8_t)e[1]; w.ez = (uint8_t)e[2];
    for (size_t k = 0; k < ch.size(); ++k) {
        for (int a = 0; a < 3; ++a) {
            const float s = wide_scale(e[a]);
            int lo = (int)std::floor((ch[k].box.lo[a] - p[a]) / s);
            int hi = (int)std::ceil((ch[k].box.hi[a] - p[a]) / s);
            lo = std::min(std::max(lo, 0), 255);
            hi = std::min(std::max(hi, 0), 255);
            while (lo > 0 && wide_plane(p[a], lo, s) > ch[k].box.lo[a]) --lo;
            while (hi < 255 && wide_plane(p[a], hi, s) < ch[k].box.hi[a]) ++hi;
            w.qlo[a][k] = (uint8_t)lo;
            w.qhi[a][k] = (uint8_t)hi;
        }
    }
}

}  // namespace

void build_wide(const std::vector<Aabb> &boxes, int max_leaf, int node_base, int prim_base, WideOut &out) {
    BvhOut b2;
    build_bvh(boxes, max_leaf, 0, 0, b2);
    out.nodes.clear();
    out.order.clear();
    out.depth = 0;
    out.stack = 1;
    DWide empty;
    std::memset(&empty, 0, sizeof(empty));
    empty.ex = empty.ey = empty.ez = 127;
    if (boxes.empty()) {   /* no primitives: one node without children */
        out.nodes.push_back(empty);
        out.root_ref = node_base << 4;
        return;
    }
    if (b2.root_ref & 15) {   /* the whole set is one leaf */
        out.order = b2.order;
        out.nodes.push_back(empty);   /* unused placeholder keeps node numbering simple */
        out.root_ref = (prim_base << 4) | (b2.root_ref & 15);
        return;
    }
    auto children = [&](int idx, std::vector<WideCand> &v) {
        const DNode &d = b2.nodes[idx];
        WideCand a, b;
        a.box.lo[0] = d.xs.x; a.box.hi[0] = d.xs.y; a.box.lo[1] = d.ys.x; a.box.hi[1] = d.ys.y;
        a.box.lo[2] = d.zs.x; a.box.hi[2] = d.zs.y; a.ref = d.ch.x;
        b.box.lo[0] = d.xs.z; b.box.hi[0] = d.xs.w; b.box.lo[1] = d.ys.z; b.box.hi[1] = d.ys.w;
        b.box.lo[2] = d.zs.z; b.box.hi[2] = d.zs.w; b.ref = d.ch.y;
        v.push_back(a);
        v.push_back(b);
    };
    /* anc = entries a traversal can hold below this node's pushes: the sum of (children - 1) over
     * its ancestors */
    struct Item { int ref; Aabb box; int wide, depth, anc; };
    std::deque<Item> queue;
    {
        std::vector<WideCand> r;
        children(b2.root_ref >> 4, r);
        Aabb rb = r[0].box;
        grow(rb, r[1].box);
        queue.push_back({b2.root_ref, rb, 0, 1, 0});
    }
    out.nodes.push_back(empty);
    std::vector<WideCand> ch;
    while (!queue.empty()) {
        const Item it = queue.front();
        queue.pop_front();
        out.depth = std::max(out.depth, it.depth);
        ch.clear();
        children(it.ref >> 4, ch);
        while (ch.size() < 8) {   /* open the inner child of largest surface area */
            int best = -1;
            float ba = -1.f;
            for (size_t i = 0; i < ch.size(); ++i)
                if ((ch[i].ref & 15) == 0 && area(ch[i].box) > ba) { ba = area(ch[i].box); best = (int)i; }
            if (best < 0) break;
            std::vector<WideCand> sub;
            children(ch[best].ref >> 4, sub);
            ch[best] = sub[0];
            ch.insert(ch.begin() + best + 1, sub[1]);
        }
        DWide w = empty;
        w.nchild = (uint8_t)ch.size();
        out.stack = std::max(out.stack, it.anc + (int)ch.size());
        quantise(w, it.box, ch);
        const int base = (int)out.nodes.size();
        const int leaf0 = (int)out.order.size();
        w.child_base = node_base + base;
        w.leaf_base = prim_base + leaf0;
        int inner = 0;
        for (size_t k = 0; k < ch.size(); ++k) {
            if ((ch[k].ref & 15) == 0) {
                w.meta[k] = (uint8_t)(inner << 3);
                queue.push_back({ch[k].ref, ch[k].box, base + inner, it.depth + 1, it.anc + (int)ch.size() - 1});
                ++inner;
            } else {
                const int first = ch[k].ref >> 4, cnt = ch[k].ref & 15;
                w.meta[k] = (uint8_t)(((int)out.order.size() - leaf0) << 3 | cnt);
                for (int j = 0; j < cnt; ++j) out.order.push_back(b2.order[first + j]);
            }
        }
        for (int i = 0; i < inner; ++i) out.nodes.push_back(empty);
        out.nodes[it.wide] = w;
    }
    out.root_ref = node_base << 4;
}

/* ------------------------------------------------------------------ shader-graph compiler */
namespace {

struct Val { int vreg; uint8_t type; };

struct Emitter {
    const lgpu_scene_desc *d;
    const std::vector<int> *tex_off = nullptr;
    std::vector<DIns> ins;          /* SSA: instruction i writes virtual register i */
    std::map<std::pair<int, int>, Val> memo;
    std::string err;

    int emit(DIns in) { in.dst = 0; ins.push_back(in); return (int)ins.size() - 1; }
    static DIns mkins(uint8_t op) { DIns in; std::memset(&in, 0, sizeof(in)); in.op = op; return in; }
    int konst(float a, float b = 0, float c = 0, float e = 0) {
        DIns in = mkins(OP_CONST);
        in.k[0] = a; in.k[1] = b; in.k[2] = c; in.k[3] = e;
        return emit(in);
    }
    int conv(int v, uint8_t from, uint8_t to, bool illum = false) {
        if (from == to && to != ST_SPECTRUM) return v;
        if (from == ST_SPECTRUM && to == ST_SPECTRUM) return v;
        DIns in = mkins(OP_CONV);
        in.a = (uint8_t)v;   /* patched to physical registers later; vregs stored in a side table */
        in.sub = (uint8_t)((from << 4) | to);
        in.c = illum ? 1 : 0;
        const int r = emit(in);
        srcs.push_back({r, {v, -1, -1, -1}});
        return r;
    }
    /* side table: source vregs of each instruction (a, b, c, sub-as-register for MERGE) */
    struct Src { int ins; int v[4]; };
    std::vector<Src> srcs;
    int emit_src(DIns in, int a, int b = -1, int c = -1, int e = -1) {
        const int r = emit(in);
        srcs.push_back({r, {a, b, c, e}});
        return r;
    }

    static uint8_t out_type(int type, int out) {
        switch (type) {
        case LGPU_NODE_SEPARATE_XYZ: case LGPU_NODE_SEPARATE_RGBA: case LGPU_NODE_SCALAR: case LGPU_NODE_MATHS:
        case LGPU_NODE_DOT_PRODUCT: case LGPU_NODE_VECTOR_MAGNITUDE: case LGPU_NODE_PERLIN_NOISE:
        case LGPU_NODE_VALUE_NOISE: case LGPU_NODE_OCTAVE_NOISE: case LGPU_NODE_CHECKER: case LGPU_NODE_VORONOI:
            return ST_SCALAR;
        case LGPU_NODE_MERGE_XYZ: case LGPU_NODE_VECTOR3: case LGPU_NODE_SURFACE_INFO: case LGPU_NODE_VECTOR_MATHS:
        case LGPU_NODE_CROSS_PRODUCT:
            return ST_VEC3;
        case LGPU_NODE_MERGE_RGBA: case LGPU_NODE_RGB: return ST_COLOUR;
        case LGPU_NODE_VECTOR2: return ST_VEC2;
        case LGPU_NODE_SPECTRUM: case LGPU_NODE_BLACKBODY: return ST_SPECTRUM;
        case LGPU_NODE_IMAGE_TEXTURE: return out == 0 ? ST_COLOUR : ST_SCALAR;
        default: return ST_BXDF;
        }
    }
    static int noise_kind(int type) {
        switch (type) {
        case LGPU_NODE_PERLIN_NOISE: return NK_PERLIN;
        case LGPU_NODE_VALUE_NOISE: return NK_VALUE;
        case LGPU_NODE_CHECKER: return NK_CHECKER;
        case LGPU_NODE_VORONOI: return NK_VORONOI;
        case LGPU_NODE_OCTAVE_NOISE: return NK_OCTAVE;
        default: return -1;
        }
    }
    bool linked(int node, int i) const { return d->nodes[node].in_node[i] >= 0; }
    const float *def(int node, int i) const { return d->nodes[node].in_default[i]; }

    /* SocketRef::GetAs<T> of input i */
    int get_as(int node, int i, uint8_t to) {
        if (!linked(node, i)) {
            const float *v = def(node, i);
            switch (to) {
            case ST_SCALAR: return konst(v[0]);
            case ST_VEC2: return konst(v[0], v[1]);
            case ST_VEC3: return konst(v[0], v[1], v[2]);
            default: return konst(v[0], v[1], v[2], v[3]);
            }
        }
        const Val s = output(d->nodes[node].in_node[i], d->nodes[node].in_socket[i]);
        if (s.vreg < 0) return -1;
        return conv(s.vreg, s.type, to);
    }
    /* SocketRef::GetAsSpectrum of input i (reflectance). */
    int get_spectrum(int node, int i) {
        if (!linked(node, i)) {
            const float *v = def(node, i);
            const int c = konst(v[0], v[1], v[2], v[3]);
            return conv(c, ST_COLOUR, ST_SPECTRUM, false);
        }
        const Val s = output(d->nodes[node].in_node[i], d->nodes[node].in_socket[i]);
        if (s.vreg < 0) return -1;
        return spectrum_of(s, false);
    }
    /* Socket::GetAsSpectrum(type) (ShaderGraph.h:232-251) */
    int spectrum_of(Val s, bool illum) {
        switch (s.type) {
        case ST_COLOUR: return conv(s.vreg, ST_COLOUR, ST_SPECTRUM, illum);
        case ST_SCALAR: return conv(s.vreg, ST_SCALAR, ST_SPECTRUM, illum);
        case ST_SPECTRUM: return s.vreg;
        default: return konst(0, 0, 0, 0);
        }
    }

    Val output(int node, int out) {
        if (node < 0 || node >= d->num_nodes) { err = "dangling socket link"; return {-1, 0}; }
        auto it = memo.find({node, out});
        if (it != memo.end()) return it->second;
        const lgpu_node_desc &nd = d->nodes[node];
        const uint8_t t = out_type(nd.type, out);
        int r = -1;
        switch (nd.type) {
        case LGPU_NODE_SCALAR: r = konst(nd.params[0]); break;
        case LGPU_NODE_VECTOR2: r = konst(nd.params[0], nd.params[1]); break;
        case LGPU_NODE_VECTOR3: r = konst(nd.params[0], nd.params[1], nd.params[2]); break;
        case LGPU_NODE_RGB: r = konst(nd.params[0], nd.params[1], nd.params[2], 1.f); break;
        case LGPU_NODE_SPECTRUM: r = conv(konst(nd.params[0], nd.params[1], nd.params[2], 1.f), ST_COLOUR, ST_SPECTRUM, false); break;
        case LGPU_NODE_SURFACE_INFO: r = emit(mkins(OP_NORMAL)); break;
        case LGPU_NODE_IMAGE_TEXTURE: {
            const int ti = (int)nd.params[0];
            if (!tex_off || ti < 0 || ti >= d->num_textures || ti >= (int)tex_off->size()) { err = "image texture node without a scene texture"; break; }
            DIns in = mkins(OP_IMAGE);
            in.sub = (uint8_t)(out == 1 ? 1 : 0);
            in.k[0] = bits_to_float((*tex_off)[ti]);
            in.k[1] = (float)d->textures[ti].width;
            in.k[2] = (float)d->textures[ti].height;
            r = emit(in);
            break;
        }
        case LGPU_NODE_BLACKBODY: {
            const int samples = nd.params[0] > 0 ? (int)nd.params[0] : 3;
            const int src = nd.in_node[0];
            if (src >= 0 && d->nodes[src].type == LGPU_NODE_SCALAR) {
                const float T = d->nodes[src].params[0];
                float rgb[3];
                blackbody_rgb(T, samples, rgb);
                DIns in = mkins(OP_BBCONST);
                in.k[0] = rgb[0]; in.k[1] = rgb[1]; in.k[2] = rgb[2]; in.k[3] = T;
                r = emit(in);
            } else {
                const int tv = get_as(node, 0, ST_SCALAR);
                if (tv < 0) break;
                DIns in = mkins(OP_BB);
                in.k[0] = (float)samples;
                r = emit_src(in, tv);
            }
            break;
        }
        case LGPU_NODE_SEPARATE_XYZ: {   /* B14: all outputs read input 0 */
            const int v = get_as(node, 0, ST_VEC3);
            if (v < 0) break;
            DIns in = mkins(OP_SEP); in.sub = (uint8_t)out;
            r = emit_src(in, v);
            break;
        }
        case LGPU_NODE_SEPARATE_RGBA: {
            const int v = get_as(node, 0, ST_COLOUR);
            if (v < 0) break;
            DIns in = mkins(OP_SEP); in.sub = (uint8_t)out;
            r = emit_src(in, v);
            break;
        }
        case LGPU_NODE_MERGE_XYZ: {
            const int a = get_as(node, 0, ST_SCALAR), b = get_as(node, 1, ST_SCALAR), c = get_as(node, 2, ST_SCALAR);
            if (a < 0 || b < 0 || c < 0) break;
            DIns in = mkins(OP_MERGE); in.sub = 255;
            r = emit_src(in, a, b, c);
            break;
        }
        case LGPU_NODE_MERGE_RGBA: {
            const int a = get_as(node, 0, ST_SCALAR), b = get_as(node, 1, ST_SCALAR), c = get_as(node, 2, ST_SCALAR),
                      e = get_as(node, 3, ST_SCALAR);
            if (a < 0 || b < 0 || c < 0 || e < 0) break;
            DIns in = mkins(OP_MERGE);
            r = emit_src(in, a, b, c, e);
            break;
        }
        case LGPU_NODE_MATHS: {
            const int a = get_as(node, 0, ST_SCALAR);
            const int b = nd.op == LGPU_MATHS_SQRT ? a : get_as(node, 1, ST_SCALAR);
            if (a < 0 || b < 0) break;
            DIns in = mkins(OP_MATHS); in.sub = (uint8_t)nd.op;
            r = emit_src(in, a, b);
            break;
        }
        case LGPU_NODE_VECTOR_MATHS: {
            const int a = get_as(node, 0, ST_VEC3), b = get_as(node, 1, ST_VEC3);
            if (a < 0 || b < 0) break;
            DIns in = mkins(OP_VMATHS); in.sub = (uint8_t)nd.op;
            r = emit_src(in, a, b);
            break;
        }
        case LGPU_NODE_DOT_PRODUCT: case LGPU_NODE_CROSS_PRODUCT: {
            const int a = get_as(node, 0, ST_VEC3), b = get_as(node, 1, ST_VEC3);
            if (a < 0 || b < 0) break;
            r = emit_src(mkins(nd.type == LGPU_NODE_DOT_PRODUCT ? OP_DOT : OP_CROSS), a, b);
            break;
        }
        case LGPU_NODE_VECTOR_MAGNITUDE: {
            const int a = get_as(node, 0, ST_VEC3);
            if (a < 0) break;
            r = emit_src(mkins(OP_LEN), a);
            break;
        }
        case LGPU_NODE_PERLIN_NOISE: case LGPU_NODE_VALUE_NOISE: case LGPU_NODE_CHECKER: case LGPU_NODE_VORONOI: {
            DIns in = mkins(OP_NOISE); in.sub = (uint8_t)noise_kind(nd.type); in.k[0] = nd.params[0];
            r = emit(in);
            break;
        }
        case LGPU_NODE_OCTAVE_NOISE: {
            const int inner = nd.in_node[0];
            const int k = inner >= 0 ? noise_kind(d->nodes[inner].type) : -1;
            if (k < 0 || k == NK_OCTAVE) { err = "OctaveNoise needs a Perlin/Value/Checker/Voronoi noise node as input 0"; break; }
            DIns in = mkins(OP_NOISE);
            in.sub = NK_OCTAVE; in.c = (uint8_t)k;
            in.k[0] = nd.params[0]; in.k[1] = nd.params[1]; in.k[2] = d->nodes[inner].params[0];
            r = emit(in);
            break;
        }
        default:
            err = "unsupported shader node type " + std::to_string(nd.type);
            break;
        }
        const Val v{r, t};
        if (r >= 0) memo[{node, out}] = v;
        return v;
    }

    /* Linear-scan register allocation; `live_out` vregs stay live to the end.  Returns false if
     * more than `limit` registers are needed. */
    bool allocate(const std::vector<int> &live_out, int limit, std::vector<int> &phys, int &used) {
        const int n = (int)ins.size();
        std::vector<int> last(n, -1);
        std::vector<std::vector<int>> uses(n);
        for (auto &s : srcs)
            for (int k = 0; k < 4; ++k)
                if (s.v[k] >= 0) { last[s.v[k]] = std::max(last[s.v[k]], s.ins); uses[s.ins].push_back(s.v[k]); }
        for (int v : live_out) if (v >= 0) last[v] = n;
        phys.assign(n, -1);
        std::vector<int> freeUntil(limit, -1);   /* register r is busy until instruction freeUntil[r] */
        used = 0;
        for (int i = 0; i < n; ++i) {
            int r = -1;
            for (int k = 0; k < limit; ++k) if (freeUntil[k] < i) { r = k; break; }
            /* an instruction may overwrite a source that dies at this very instruction */
            if (r < 0) {
                for (int v : uses[i]) if (last[v] == i) { r = phys[v]; break; }
            }
            if (r < 0) return false;
            phys[i] = r;
            freeUntil[r] = last[i] < 0 ? i : last[i];
            used = std::max(used, r + 1);
        }
        return true;
    }
    /* Write the allocated program into `code`. */
    void finish(std::vector<DIns> &code, const std::vector<int> &phys) {
        std::vector<Src *> byIns(ins.size(), nullptr);
        for (auto &s : srcs) byIns[s.ins] = &s;
        for (size_t i = 0; i < ins.size(); ++i) {
            DIns in = ins[i];
            in.dst = (uint8_t)phys[i];
            if (byIns[i]) {
                const Src &s = *byIns[i];
                if (s.v[0] >= 0) in.a = (uint8_t)phys[s.v[0]];
                if (s.v[1] >= 0) in.b = (uint8_t)phys[s.v[1]];
                if (s.v[2] >= 0) in.c = (uint8_t)phys[s.v[2]];
                if (s.v[3] >= 0) in.sub = (uint8_t)phys[s.v[3]];
            }
            code.push_back(in);
        }
    }
};

}  // namespace

bool GraphCompiler::compile_material(int bxdf_node, DMaterial &m) {
    Emitter E;
    E.d = d;
    E.tex_off = tex_off;
    m.num_leaves = 0;
    m.num_tree = 0;
    struct LeafV { int alb, rough; };
    std::vector<LeafV> lv;
    std::vector<int> ratioV;
    /* tree slots: preorder, slot 0 = root */
    std::function<int(int, int)> walk = [&](int node, int depth) -> int {
        if (node < 0 || node >= d->num_nodes) { err = "material BxDF link is dangling"; return -1; }
        const lgpu_node_desc &nd = d->nodes[node];
        const int slot = m.num_tree++;
        if (slot >= 2 * LGPU_MAX_LEAVES - 1) { err = "BSDF mix tree too large"; return -1; }
        ratioV.resize(m.num_tree, -1);
        if (nd.type == LGPU_NODE_BXDF_MIX) {
            if (depth >= 2) { err = "Mix BSDF nesting deeper than 2"; return -1; }
            m.tree[slot].kind = 1;
            const int r = E.get_as(node, 2, ST_SCALAR);
            ratioV[slot] = r;
            const int a = walk(nd.in_node[0], depth + 1);
            if (a < 0) return -1;
            const int b = walk(nd.in_node[1], depth + 1);
            if (b < 0) return -1;
            m.tree[slot].a = (uint8_t)a;
            m.tree[slot].b = (uint8_t)b;
            return slot;
        }
        if (m.num_leaves >= LGPU_MAX_LEAVES) { err = "more than 4 BSDF lobes"; return -1; }
        const int li = m.num_leaves++;
        DLeaf &L = m.leaves[li];
        std::memset(&L, 0, sizeof(L));
        L.type = (uint8_t)nd.type;
        LeafV v{-1, -1};
        switch (nd.type) {
        case LGPU_NODE_BXDF_LAMBERTIAN:
            v.alb = E.get_spectrum(node, 0);
            break;
        case LGPU_NODE_BXDF_OREN_NAYAR_R: case LGPU_NODE_BXDF_OREN_NAYAR_T:
        case LGPU_NODE_BXDF_FRESNEL:
            v.alb = E.get_spectrum(node, 0);
            v.rough = E.get_as(node, 1, ST_SCALAR);
            break;
        case LGPU_NODE_BXDF_MICROFACET_R:
            v.alb = E.get_spectrum(node, 0);
            v.rough = E.get_as(node, 1, ST_SCALAR);
            L.dist = (uint8_t)nd.params[0];
            L.eta = nd.params[1];
            break;
        case LGPU_NODE_BXDF_SPECULAR_R:
            v.alb = E.get_spectrum(node, 0);
            break;
        default:
            err = "unsupported BxDF node type " + std::to_string(nd.type);
            return -1;
        }
        lv.push_back(v);
        m.tree[slot].kind = 0;
        m.tree[slot].a = (uint8_t)li;
        return slot;
    };
    if (walk(bxdf_node, 0) < 0) return false;
    if (!E.err.empty()) { err = E.err; return false; }
    std::vector<int> live;
    for (auto &v : lv) { live.push_back(v.alb); live.push_back(v.rough); }
    for (int r : ratioV) live.push_back(r);
    std::vector<int> phys;
    int used = 0;
    if (!E.allocate(live, LGPU_MAX_REGS, phys, used)) { err = "shader graph needs more than 16 registers"; return false; }
    m.prog_off = (int)code->size();
    E.finish(*code, phys);
    m.prog_len = (int)code->size() - m.prog_off;
    /* registers of leaf inputs; a missing value reads a zero constant register */
    for (int i = 0; i < m.num_leaves; ++i) {
        m.leaves[i].albedo = (uint8_t)(lv[i].alb >= 0 ? phys[lv[i].alb] : 0);
        m.leaves[i].rough = (uint8_t)(lv[i].rough >= 0 ? phys[lv[i].rough] : 0);
    }
    for (int i = 0; i < m.num_tree; ++i) m.tree[i].ratio = (uint8_t)(ratioV[i] >= 0 ? phys[ratioV[i]] : 0);
    fold_material(m);
    return true;
}

/* Does a program read the shading event (uv, point, normal, noise, Fresnel input)? */
bool GraphCompiler::context_free(int off, int len) const {
    for (int i = 0; i < len; ++i) {
        const uint8_t op = (*code)[off + i].op;
        if (op == OP_UV || op == OP_POINT || op == OP_NORMAL || op == OP_NOISE || op == OP_SCHLICK || op == OP_IMAGE) return false;
    }
    return true;
}

/* RGB mode: evaluate a context-free material program once, here. */
void GraphCompiler::fold_material(DMaterial &m) {
    m.folded = 0;
    if (!context_free(m.prog_off, m.prog_len)) return;
    float4 R[LGPU_MAX_REGS];
    std::memset(R, 0, sizeof(R));
    ShadeCtx ctx;
    std::memset(&ctx, 0, sizeof(ctx));
    ctx.eta = 1.001f;
    Lambda4 lam;
    std::memset(&lam, 0, sizeof(lam));
    run_prog<3>(code->data() + m.prog_off, m.prog_len, ctx, lam, R);
    for (int i = 0; i < m.num_leaves; ++i) { m.kalb[i] = R[m.leaves[i].albedo]; m.kalb[i].w = 0.f; m.krough[i] = R[m.leaves[i].rough].x; }
    for (int i = 0; i < m.num_tree; ++i) m.kratio[i] = m.tree[i].kind ? R[m.tree[i].ratio].x : 0.f;
    m.folded = 1;
}

bool GraphCompiler::compile_emission(int node, int socket, int &prog_off, int &prog_len, int &out_reg) {
    Emitter E;
    E.d = d;
    E.tex_off = tex_off;
    const Val v = E.output(node, socket);
    if (v.vreg < 0 || !E.err.empty()) { err = E.err.empty() ? "bad emission socket" : E.err; return false; }
    const int illum = E.spectrum_of(v, true);
    const int refl = E.spectrum_of(v, false);
    std::vector<int> phys;
    int used = 0;
    if (!E.allocate({illum, refl}, LGPU_MAX_REGS - 2, phys, used)) { err = "emission graph needs too many registers"; return false; }
    prog_off = (int)code->size();
    E.finish(*code, phys);
    /* copy the two results into consecutive registers `used`, `used + 1` via a neutral conversion */
    out_reg = used;
    DIns c1 = Emitter::mkins(OP_CONV);
    c1.a = (uint8_t)phys[illum]; c1.sub = (uint8_t)((ST_SPECTRUM << 4) | ST_SPECTRUM); c1.dst = (uint8_t)used;
    DIns c2 = c1;
    c2.a = (uint8_t)phys[refl]; c2.dst = (uint8_t)(used + 1);
    code->push_back(c1);
    code->push_back(c2);
    prog_len = (int)code->size() - prog_off;
    return true;
}

/* RGB mode: evaluate a context-free emission program once; returns false if it reads the event. */
bool GraphCompiler::fold_emission(int prog_off, int prog_len, int out_reg, float4 em[2]) {
    if (!context_free(prog_off, prog_len)) return false;
    float4 R[LGPU_MAX_REGS];
    std::memset(R, 0, sizeof(R));
    ShadeCtx ctx;
    std::memset(&ctx, 0, sizeof(ctx));
    ctx.eta = 1.001f;
    Lambda4 lam;
    std::memset(&lam, 0, sizeof(lam));
    run_prog<3>(code->data() + prog_off, prog_len, ctx, lam, R);
    em[0] = R[out_reg]; em[0].w = 0.f;
    em[1] = R[out_reg + 1]; em[1].w = 0.f;
    return true;
}

}  // namespace lg
