/*
 * Device-resident scene layout of the GB300 path tracer (host/device shared definitions).
 *
 * Everything a kernel reads lives in a handful of flat arrays in HBM, addressed by 32-bit
 * indices, so one launch can hold ~100 M instanced triangles without per-object pointers:
 *
 *   BVH nodes   DNode  64 B  binary node: both child boxes + child refs (default), or
 *               DWide  80 B  8-wide node: eight child boxes quantised to 8 bits per plane against
 *                            the node box, child records consecutive (built with LGPU_BVH_WIDE=1)
 *   triangles   DTri   48 B  v0, e1 = v1 - v0, e2 = v2 - v0 (Moller-Trumbore form), prim and
 *                            object ids in the w lanes; leaf triangles are contiguous
 *   instances   DInst  64 B  world->object 3x4 affine + BLAS root (TLAS leaves)
 *   objects     DObject      Lambda Scene::objects: mesh, material, linear part + normal matrix
 *   meshes      DMesh        offsets into the vertex-attribute arrays
 *   materials   DMaterial    Material{bxdf, light, mediaBoundary}; bxdf is a compiled program
 *   programs    DIns         shader-graph bytecode, one linear program per graph root
 *   lights      DLight       Light table; light-tree nodes DLNode; leaf CDFs in a float pool
 */
#pragma once
#include <stdint.h>
#include <vector_types.h>

#define LGPU_MAX_REGS 16
#define LGPU_MAX_LEAVES 4
/* traversal stack entries; the host computes each scene's exact worst case and refuses scenes
 * above it */
#define LGPU_STACK 96
/* Node layout of the device BVH: 0 = binary nodes (DNode), 1 = 8-wide compressed nodes (DWide).
 * The wide layout visits 2.7x fewer nodes on the 1080p terrain, but its traversal issues ~6x more
 * instructions per visit with 8 of 32 lanes active, and measured slower there (193 vs 168 ms of
 * traversal per frame; about even on the instanced volume scene), so binary nodes are the default. */
#ifndef LGPU_BVH_WIDE
#define LGPU_BVH_WIDE 0
#endif
/* Binary-node slab distances as one fused multiply-add per plane, fma(plane, 1/d, -o/d), instead of
 * (plane - o) * (1/d) (two roundings, two instructions without contraction). */
#ifndef LGPU_BOX_FMA
#define LGPU_BOX_FMA 0
#endif

/* BVH2 node (binned SAH build): child c's box is (xs[2c], xs[2c+1]) etc.
 * ch = (ref0, ref1, -, -): ref = (index << 4) | count, count 0 for an inner node, else the first
 * primitive record of a leaf of `count` primitives. */
struct DNode {
    float4 xs, ys, zs;
    int4 ch;
};

/* 8-wide BVH node, 80 bytes (five 16-byte loads).  The node box's minimum corner p and per-axis
 * power-of-two scales s = 2^(e - 127) define the child boxes: child k spans
 * [p + qlo[a][k] * s_a, p + qhi[a][k] * s_a] on axis a.  The product q * s is exact, so host and
 * device decode the same floats, and the builder rounds every plane outwards (the decoded box
 * contains the child's true box).  Inner children are consecutive node records from child_base;
 * leaf children's primitives are consecutive records from leaf_base.  meta[k]: bits 0-2 = the
 * leaf's primitive count (0 for an inner child), bits 3-7 = offset from child_base (inner) or
 * leaf_base (leaf).  Children k >= nchild are absent. */
struct __align__(16) DWide {
    float px, py, pz;
    uint8_t ex, ey, ez, nchild;
    int child_base, leaf_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(DWide) == 80, "DWide must be 80 bytes");
#if LGPU_BVH_WIDE
typedef DWide BvhNode;
#else
typedef DNode BvhNode;
#endif

struct DTri {
    float4 v0;   /* w = prim id (bits) */
    float4 e1;   /* w = object id (bits) */
    float4 e2;   /* w = unused */
};

struct DInst {
    float4 r0, r1, r2;   /* rows of the object's inverse linear part; w = the object's translation t
                          * (world -> object: inv * (x - t)) */
    int root;            /* BLAS root node */
    int object;          /* object id written into hits (-1: per-triangle object ids) */
    int pad0, pad1;
};

struct DObject {
    int mesh, material, kind, identity;
    float m[9];     /* column-major linear part (object -> world) */
    float nrm[9];   /* column-major inverse transpose (normal matrix) */
    float t[3];
    float pad;
};

struct DMesh {
    int vtx_off;    /* into pos / nrm / tan / uv arrays */
    int tri_off;    /* into tri_idx */
    int num_tris;
    int flags;      /* 1 = smooth normals+tangents, 2 = uvs */
};

/* Bytecode instruction (24 bytes).  dst/a/b/c are register indices, k are immediates. */
struct DIns {
    uint8_t op, dst, a, b;
    uint8_t c, sub, pad0, pad1;
    float k[4];
};

/* BSDF tree of one material: up to 4 leaves under up to 3 Mix nodes.
 * tree[i]: kind 0 = leaf (idx = leaf index), kind 1 = mix (a, b = tree slots, ratio register). */
struct DLeaf {
    uint8_t type;        /* lgpu_node_type of the BxDF node */
    uint8_t albedo;      /* register holding the albedo spectrum */
    uint8_t rough;       /* register holding roughness / sigma / ior (x) */
    uint8_t dist;        /* microfacet distribution */
    float eta;           /* FresnelDielectric etaT of microfacet lobes */
};
struct DBsdfNode {
    uint8_t kind, a, b, ratio;
};
struct DMaterial {
    int prog_off, prog_len;      /* shader program computing the leaf inputs (-1: none) */
    int light;                   /* light index or -1 */
    int medium_interior, medium_exterior;
    int has_bsdf;
    int num_leaves, num_tree;
    DLeaf leaves[LGPU_MAX_LEAVES];
    DBsdfNode tree[2 * LGPU_MAX_LEAVES - 1];
    int folded;                  /* RGB mode: graph is context-free, constants below are its values */
    float4 kalb[LGPU_MAX_LEAVES];
    float krough[LGPU_MAX_LEAVES];
    float kratio[2 * LGPU_MAX_LEAVES - 1];
};

enum { LT_POINT = 0, LT_MESH = 1, LT_ENV = 2, LT_SPOT = 3, LT_TRI = 4 };

struct DLight {
    int type;
    int prog_off, prog_len, out_reg;   /* emission program and its output register */
    int object;                        /* emitting object (mesh lights) */
    int dist_off;                      /* mesh lights: triangle-area CDF (n+1) then areas (n) in fpool */
    int num_tris;
    int tri_base;                      /* first tree-light index of this mesh light's triangles */
    float intensity;
    float cosCone, cosFall;
    float integral;                    /* CDF integral of the triangle distribution */
    float3 pos;
    float3 axis;
    float power;
    int em_folded;                     /* RGB mode: emission graph is context-free */
    float4 em[2];                      /* its illuminant and reflectance spectra */
};

/* Flattened ManyLightSampler node (ManyLightSampler.h:47-60), 64 bytes.  Bounds are stored as the
 * centre and diagonal length the importance measure uses (Bounds::Center / DiagonalLength,
 * evaluated on the host with the reference's float operations).  Children are consecutive records
 * (child1 = child0 + 1) and sibling pairs start on a 128-byte boundary, so one line fetch serves
 * both importance evaluations of a descent step.  Record 0 is unused; the root is record 1. */
struct __align__(16) DLNode {
    float3 center;
    float diag;
    float3 axis;
    float cosO;          /* cos / sin of the orientation-cone angle thetaO; every node's emission */
    float sinO, power;   /* angle thetaE is pi/2 (MakeCone's default, kept by OrientationCone::Union) */
    int child0, parent;
    int first, num;      /* light range in tree order */
    int dist_off;        /* leaf: CDF (num+1) then raw powers (num) in fpool */
    float integral;      /* leaf CDF integral */
};

struct DMedium {
    float sa[4], ss[4];
    float g;
    float pad[3];
};

struct DEnv {
    int w, h;
    int present;
    float intensity;
    float offx, offy;
    float marg_integral;
    int tex_off;        /* float4 texels in env_tex */
    int marg_off;       /* fpool: marginal CDF (h+1), marginal func (h) */
    int cond_off;       /* fpool: per row: CDF (w+1), func (w), integral (1) */
};

struct DeviceScene {
    const BvhNode *nodes;
    const DTri *tris;
    const DInst *insts;
    const DObject *objects;
    const DMesh *meshes;
    const float4 *pos;
    const float4 *nrm;
    const float4 *tan;
    const float2 *uv;
    const uint4 *tri_idx;
    const DMaterial *materials;
    const DIns *prog;
    const DLight *lights;
    const DLNode *lnodes;
    const int2 *tree_lights;     /* (light, tri) in tree order; tri = -1 for non-mesh lights */
    const int2 *tree_slot;       /* per tree-light index: (leaf node, slot) */
    const int *light_slot;       /* per light (non-mesh): tree-light index */
    const float *fpool;
    const float4 *env_tex;
    const DMedium *media;
    DEnv env;
    int root;                    /* TLAS root (use_tlas) or world BLAS root */
    int use_tlas;
    int num_lights;
    int light_strategy;          /* 0 power, 1 tree */
    int power_cdf_off;           /* power sampler: CDF (n+1), func (n) */
    float power_integral;
    float inv_total_power;
    int tree_root;
    int num_tree_lights;
    float tree_power, inf_power;
    int env_light;               /* light index of the environment light or -1 */
    int has_volumes;
    int *err;                    /* device error word of the context (bits: traversal stack overflow,
                                  * path-state staging wait ran out), read and cleared by the host */
};
