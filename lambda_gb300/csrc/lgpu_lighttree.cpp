/*
 * Light-tree construction for the GPU light sampler (ManyLightSampler::Commit, InitLights,
 * RecursiveBuild, SplitAxis, SAOH, MOmega and OrientationCone::Union --
 * src/lighting/ManyLightSampler.cpp:37-303).  The tree is built on the host with the reference's
 * float arithmetic step for step -- 12 SAOH buckets, orientation-cone unions (including the
 * in-place operand swap of OrientationCone::Union), std::partition -- and flattened into DLNode
 * records with parent links and leaf power CDFs, so the device can sample and evaluate pdfs
 * without pointers or hash maps.
 * Compiled with -ffp-contract=off so Arm and x86 hosts produce the same tree.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include <cuda_runtime.h>

#include "lgpu_lighttree.h"

namespace lg {
namespace lt {

static const float PIf = 3.14159265358979323846f;
static const float PI2f = 2.0f * 3.14159265358979323846f;

static inline float fmin_(float a, float b) { return std::min(a, b); }
static inline float fmax_(float a, float b) { return std::max(a, b); }
static inline float clampf_(float v, float lo, float hi) { return std::max(std::min(v, hi), lo); }

V3f operator+(V3f a, V3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3f operator-(V3f a, V3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3f operator*(V3f a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline float dot(V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3f cross(V3f a, V3f b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline float mag(V3f a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline float comp(V3f a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

Box Box::unite(const Box &a, const Box &b) {
    Box r;
    r.mn = {std::min(a.mn.x, b.mn.x), std::min(a.mn.y, b.mn.y), std::min(a.mn.z, b.mn.z)};
    r.mx = {std::max(a.mx.x, b.mx.x), std::max(a.mx.y, b.mx.y), std::max(a.mx.z, b.mx.z)};
    return r;
}
float Box::surface() const { const V3f s = mx - mn; return (s.x * s.y + s.y * s.z + s.x * s.z) * 2.f; }
V3f Box::center() const { return mn + (mx - mn) * .5f; }
float Box::diagonal() const { return mag(mx - mn); }
V3f Box::offset(V3f p) const { const V3f o = p - mn, d = mx - mn; return {o.x / d.x, o.y / d.y, o.z / d.z}; }

/* Rodrigues rotation with the reference's unnormalised axis (src/maths/vec3.h:230-234). */
static V3f rotate(V3f v, V3f axis, float theta) {
    const float c = std::cos(theta);
    const float s = std::sqrt(1.f - c * c);
    return v * c + cross(axis, v) * s + axis * dot(axis, v) * (1.f - c);
}
static Cone make_cone(V3f axis) { Cone c; c.axis = axis; c.thetaO = 0; c.thetaE = PIf / 2.f; return c; }
/* OrientationCone::Union (ManyLightSampler.cpp:50-64): swaps its operands in place when b is wider. */
static Cone cone_union(Cone *a, Cone *b) {
    if (b->thetaO > a->thetaO) std::swap(*a, *b);
    const float thetaE = std::max(a->thetaE, b->thetaE);
    const float thetaD = std::acos(clampf_(dot(a->axis, b->axis), 0.f, 1.f));
    Cone r;
    if (std::min(thetaD + b->thetaO, PIf) <= a->thetaO) { r.axis = a->axis; r.thetaO = a->thetaO; r.thetaE = thetaE; return r; }
    const float thetaO = (a->thetaO + thetaD + b->thetaO) * .5f;
    if (thetaO >= PIf) { r.axis = a->axis; r.thetaO = PIf; r.thetaE = thetaE; return r; }
    const float thetaR = thetaO - a->thetaO;
    r.axis = rotate(a->axis, cross(a->axis, b->axis), thetaR);
    r.thetaO = thetaO;
    r.thetaE = thetaE;
    return r;
}
static Cone cone_union_v(Cone a, Cone b) { return cone_union(&a, &b); }
static float momega(const Cone &c) {   /* :71-78 */
    const float cosO = std::cos(c.thetaO);
    const float sinO = std::sqrt(1 - cosO * cosO);
    const float a = PI2f * (1.f - cosO);
    const float thetaW2 = std::min(c.thetaO + c.thetaE, PIf) * 2.f;
    const float b = thetaW2 * sinO - std::cos(c.thetaO - thetaW2) - 2.f * c.thetaO * sinO + cosO;
    return a + PIf * .5f * b;
}
static unsigned to_unsigned(float x) {   /* float -> unsigned as x86-64 code converts it */
    if (!(x == x) || std::isinf(x) || x >= 9.2e18f || x <= -9.2e18f) return 0u;
    return (unsigned)(uint64_t)(int64_t)x;
}

namespace {
struct Node {
    int ch[2] = {-1, -1};
    int parent = -1;
    unsigned first = 0, num = 0;
    Box b;
    Cone cone;
    float power = 0, var = 0;
    std::vector<float> leafPowers;
};
struct Bucket { float power = 0; Box b; Cone cone; };

struct Builder {
    std::vector<int> order;              /* tree-light indices in tree order */
    const std::vector<TreeLightIn> *in;
    std::vector<Node> nodes;
    float treePower = 0;
    const TreeLightIn &L(unsigned i) const { return (*in)[order[i]]; }

    float power_variance(unsigned first, unsigned n) const {
        std::vector<float> p(n);
        float mean = 0;
        for (unsigned i = 0; i < n; ++i) { p[i] = L(i + first).power; mean += p[i]; }
        mean /= (float)n;
        float sum = 0;
        for (unsigned i = 0; i < n; ++i) { const float t = p[i] - mean; sum += t * t; }
        return sum / (float)(n - 1);
    }
    static float saoh(const Node &P, const Bucket &R, const Bucket &Lb, unsigned axis) {
        const V3f box = P.b.mx - P.b.mn;
        const float lenMax = std::max(std::max(box.x, box.y), box.z);
        const float Kr = lenMax / comp(box, (int)axis);
        const float m = P.b.surface() * momega(P.cone);
        const float mL = Lb.power * Lb.b.surface() * momega(Lb.cone);
        const float mR = R.power * R.b.surface() * momega(R.cone);
        return Kr * (mL + mR) / m;
    }
    void init_leaf(int ni) {
        Node &n = nodes[ni];
        n.leafPowers.resize(n.num);
        for (unsigned i = 0; i < n.num; ++i) {
            n.leafPowers[i] = L(n.first + i).power;
            treePower += n.leafPowers[i];
        }
        n.ch[0] = n.ch[1] = -1;
    }
    bool split_axis(int ni, unsigned axis, float *minCost, unsigned *bi, Bucket *lb, Bucket *rb) {
        const unsigned NB = 12;
        Bucket bk[NB];
        bool init[NB] = {false};
        const Node &n = nodes[ni];
        for (unsigned i = n.first; i < n.first + n.num; ++i) {
            const TreeLightIn &l = L(i);
            unsigned b = to_unsigned((float)NB * comp(n.b.offset(l.b.center()), (int)axis));
            if (b == NB) b = NB - 1;
            if (b > NB) b = 0;
            if (!init[b]) { bk[b].power = l.power; bk[b].b = l.b; bk[b].cone = make_cone(l.dir); init[b] = true; }
            else {
                bk[b].power += l.power;
                bk[b].b = Box::unite(bk[b].b, l.b);
                bk[b].cone = cone_union_v(bk[b].cone, make_cone(l.dir));
            }
        }
        bool cheaper = false;
        for (unsigned i = 0; i < NB - 1; ++i) {
            Bucket bL; bL.power = 0; bL.b = bk[0].b; bL.cone = bk[0].cone;
            Bucket bR; bR.power = 0; bR.b = bk[i + 1].b; bR.cone = bk[i + 1].cone;
            for (unsigned j = 0; j <= i; ++j) { bL.b = Box::unite(bL.b, bk[j].b); bL.cone = cone_union(&bL.cone, &bk[j].cone); bL.power += bk[j].power; }
            for (unsigned j = i + 1; j < NB; ++j) { bR.b = Box::unite(bR.b, bk[j].b); bR.cone = cone_union(&bR.cone, &bk[j].cone); bR.power += bk[j].power; }
            const float cost = saoh(nodes[ni], bR, bL, axis);
            if (cost < *minCost) { *minCost = cost; *lb = bL; *rb = bR; *bi = i; cheaper = true; }
        }
        return cheaper;
    }
    void build(int ni) {
        {
            Node &n = nodes[ni];
            n.b = L(n.first).b;
            n.cone = make_cone(L(n.first).dir);
            for (unsigned i = 0; i < n.num; ++i) {
                n.b = Box::unite(n.b, L(i + n.first).b);
                n.cone = cone_union_v(n.cone, make_cone(L(i + n.first).dir));
            }
        }
        Bucket lb, rb;
        float minCost = std::numeric_limits<float>::infinity();
        unsigned bi = 0;
        int axis = -1;
        for (int i = 0; i < 3; ++i)
            if (split_axis(ni, (unsigned)i, &minCost, &bi, &lb, &rb)) axis = i;
        const Node n = nodes[ni];
        if (n.num > 1 && minCost < n.power) {
            auto pred = [&](int li) {
                unsigned b = to_unsigned(comp(n.b.offset((*in)[li].b.center()), axis) * 12.f);
                if (b == 12) b--;
                return b <= bi;
            };
            int *beg = &order[n.first];
            int *it = std::partition(beg, beg + n.num, pred);
            const unsigned pivot = (unsigned)(it - &order[0]);
            const unsigned ln = pivot - n.first, rn = n.num - ln;
            if (ln != 0 && rn != 0) {
                Node Ln, Rn;
                Ln.parent = ni; Ln.first = n.first; Ln.num = ln; Ln.b = lb.b; Ln.cone = lb.cone; Ln.power = lb.power;
                Ln.var = power_variance(n.first, ln);
                Rn.parent = ni; Rn.first = pivot; Rn.num = rn; Rn.b = rb.b; Rn.cone = rb.cone; Rn.power = rb.power;
                Rn.var = power_variance(pivot, rn);
                const int li = (int)nodes.size();
                nodes.push_back(Ln);
                const int ri = (int)nodes.size();
                nodes.push_back(Rn);
                nodes[ni].ch[0] = li;
                nodes[ni].ch[1] = ri;
                build(li);
                build(ri);
            } else init_leaf(ni);
        } else init_leaf(ni);
    }
};
}  // namespace

/* Piecewise1D (src/sampling/Piecewise.cpp:9-24): CDF (n + 1) then the raw function (n). */
float piecewise1d(const float *f, unsigned n, std::vector<float> &pool, int &off) {
    off = (int)pool.size();
    std::vector<float> cdf(n + 1);
    cdf[0] = 0;
    for (unsigned i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / n;
    const float integral = cdf[n];
    if (integral == 0) { for (unsigned i = 1; i < n + 1; ++i) cdf[i] = float(i) / float(n); }
    else { for (unsigned i = 1; i < n + 1; ++i) cdf[i] /= integral; }
    pool.insert(pool.end(), cdf.begin(), cdf.end());
    pool.insert(pool.end(), f, f + n);
    return integral;
}

void build_light_tree(const std::vector<TreeLightIn> &lights, std::vector<float> &pool, TreeOut &out) {
    out.nodes.clear();
    out.order.clear();
    out.tree_power = 0;
    if (lights.empty()) { out.root = -1; return; }
    Builder B;
    B.in = &lights;
    B.order.resize(lights.size());
    for (size_t i = 0; i < lights.size(); ++i) B.order[i] = (int)i;
    Node root;
    root.num = (unsigned)lights.size();
    root.first = 0;
    root.b = lights[0].b;
    root.power = 0;
    root.var = 0;
    root.cone = make_cone(lights[0].dir);
    for (unsigned i = 0; i < root.num; ++i) {
        root.b = Box::unite(root.b, lights[i].b);
        root.cone = cone_union_v(root.cone, make_cone(lights[i].dir));
        root.power += lights[i].power;
    }
    B.nodes.push_back(root);
    B.treePower = 0;
    B.build(0);
    out.tree_power = B.treePower;
    out.order = B.order;
    /* record k + 1 holds builder node k (record 0 unused): sibling pairs (2j+1, 2j+2) of the builder
     * become records (2j+2, 2j+3), a 128-byte aligned pair */
    out.root = 1;
    out.nodes.resize(B.nodes.size() + 1);
    std::memset(&out.nodes[0], 0, sizeof(DLNode));
    out.nodes[0].child0 = -1;
    out.nodes[0].parent = -1;
    for (size_t i = 0; i < B.nodes.size(); ++i) {
        const Node &n = B.nodes[i];
        DLNode d;
        const V3f c = n.b.center();
        d.center = make_float3(c.x, c.y, c.z);
        d.diag = n.b.diagonal();
        d.axis = make_float3(n.cone.axis.x, n.cone.axis.y, n.cone.axis.z);
        d.cosO = std::cos(n.cone.thetaO);
        d.sinO = std::sin(n.cone.thetaO);
        d.power = n.power;
        if (n.cone.thetaE != PIf / 2.f) { out.root = -2; return; }   /* invariant of the reference's cones */
        d.child0 = n.ch[0] >= 0 ? n.ch[0] + 1 : -1;
        d.parent = n.parent >= 0 ? n.parent + 1 : -1;
        d.first = (int)n.first;
        d.num = (int)n.num;
        d.dist_off = -1;
        d.integral = 0;
        if (n.ch[0] >= 0 && n.ch[1] != n.ch[0] + 1) { out.root = -1; return; }   /* builder invariant */
        if (n.ch[0] < 0) d.integral = piecewise1d(n.leafPowers.data(), n.num, pool, d.dist_off);
        out.nodes[i + 1] = d;
    }
}

}  // namespace lt
}  // namespace lg
