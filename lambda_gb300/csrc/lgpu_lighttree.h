/* Host light-tree builder interface (see lgpu_lighttree.cpp). */
#pragma once
#include <stdint.h>
#include <vector>
#include "lgpu_scene.h"

namespace lg {
namespace lt {

struct V3f { float x = 0, y = 0, z = 0; };
V3f operator+(V3f a, V3f b);
V3f operator-(V3f a, V3f b);
V3f operator*(V3f a, float s);

/* bounds<Real>; default-constructed bounds are the origin box (src/maths/bounds.h:12-15) */
struct Box {
    V3f mn, mx;
    static Box unite(const Box &a, const Box &b);
    float surface() const;
    V3f center() const;
    float diagonal() const;
    V3f offset(V3f p) const;
};
struct Cone { V3f axis = {0, 1, 0}; float thetaO = 0, thetaE = 0; };

/* One light of the tree (TriangleLight / PointLight / Spotlight). */
struct TreeLightIn {
    Box b;          /* Light::GetBounds */
    V3f dir;        /* Light::GetDirection */
    float power;    /* Light::Power = Irradiance * Area */
};
struct TreeOut {
    std::vector<DLNode> nodes;
    std::vector<int> order;   /* tree order -> input light index */
    int root = -1;
    float tree_power = 0;
};

void build_light_tree(const std::vector<TreeLightIn> &lights, std::vector<float> &pool, TreeOut &out);
/* Piecewise1D CDF (n+1) + raw function (n) appended to pool; returns the integral. */
float piecewise1d(const float *f, unsigned n, std::vector<float> &pool, int &off);

}  // namespace lt
}  // namespace lg
