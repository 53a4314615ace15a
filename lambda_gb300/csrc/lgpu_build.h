/*
 * Host-side scene compilation for the GB300 path tracer: BVH2 construction (binned SAH), the
 * light-tree build of ManyLightSampler and the shader-graph compiler.  Internal to the module.
 */
#pragma once
#include <string>
#include <vector>
#include "lgpu_scene.h"
#include "../../include/lambda_gpu.h"

namespace lg {

struct Aabb {
    float lo[3], hi[3];
};

/* Binned-SAH BVH2 over primitive boxes.  Output nodes are numbered from 0 (the root); child refs are
 * encoded (index << 4) | count with count 0 for inner nodes.  `order` receives the primitive order of
 * the leaves; leaf first indices point into that order plus `prim_base`. */
struct BvhOut {
    std::vector<DNode> nodes;
    std::vector<uint32_t> order;
    int root_ref = 0;
    int max_depth = 0;
};
void build_bvh(const std::vector<Aabb> &boxes, int max_leaf, int node_base, int prim_base, BvhOut &out);

/* The BVH2 collapsed into 8-wide nodes (each node takes its two children, then repeatedly opens
 * the inner child of largest surface area until it holds eight or only leaves), child boxes
 * quantised outwards to 8 bits.  Node records are numbered from node_base, primitive order from
 * prim_base: `order` lists the primitives so that each node's leaf primitives are consecutive.
 * root_ref encodes the root like a child ref; depth is the number of node levels.  stack is the
 * most entries a traversal of this tree alone can hold: the maximum over nodes of the node's child
 * count plus (children - 1) summed over its ancestors (a traversal starts with the root pushed,
 * each popped node pushes at most all its children, a popped leaf pushes nothing). */
struct WideOut {
    std::vector<DWide> nodes;
    std::vector<uint32_t> order;
    int root_ref = 0;
    int depth = 0;
    int stack = 1;
};
void build_wide(const std::vector<Aabb> &boxes, int max_leaf, int node_base, int prim_base, WideOut &out);

/* The device BVH of the compiled layout (LGPU_BVH_WIDE): nodes, primitive order, root ref and
 * node-level depth. */
struct DeviceBvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;
    int root_ref = 0;
    int depth = 0;
};
inline void build_device_bvh(const std::vector<Aabb> &boxes, int max_leaf, int node_base, int prim_base, DeviceBvh &out) {
#if LGPU_BVH_WIDE
    WideOut w;
    build_wide(boxes, max_leaf, node_base, prim_base, w);
    out.nodes.swap(w.nodes); out.order.swap(w.order); out.root_ref = w.root_ref; out.depth = w.depth;
#else
    BvhOut b;
    build_bvh(boxes, max_leaf, node_base, prim_base, b);
    out.nodes.swap(b.nodes); out.order.swap(b.order); out.root_ref = b.root_ref; out.depth = b.max_depth;
#endif
}

/* Linear BVH built on the device (Morton codes, sort, radix tree, bottom-up boxes), written as
 * binary nodes with one primitive per leaf in the numbering of build_bvh.  Needs >= 2 boxes and a
 * current CUDA device; *device_ms receives the device time.  Returns 0 or an error code (err). */
int build_lbvh_device(const std::vector<Aabb> &boxes, int node_base, int prim_base, BvhOut &out, float *device_ms,
                      std::string &err);

/* Shader-graph compiler: DAG -> linear bytecode with one register per live value. */
struct GraphCompiler {
    const lgpu_scene_desc *d = nullptr;
    std::vector<DIns> *code = nullptr;
    const std::vector<int> *tex_off = nullptr;   /* texel-pool offset of each scene texture */
    std::string err;
    /* compile the BSDF of a material into m (program appended to *code) */
    bool compile_material(int bxdf_node, DMaterial &m);
    /* compile a light's emission socket; out_reg receives the illuminant spectrum register,
     * out_reg + 1 the reflectance one */
    bool compile_emission(int node, int socket, int &prog_off, int &prog_len, int &out_reg);
    /* RGB-mode constant folding of context-free programs */
    bool context_free(int off, int len) const;
    void fold_material(DMaterial &m);
    bool fold_emission(int prog_off, int prog_len, int out_reg, float4 em[2]);
};

}  // namespace lg
