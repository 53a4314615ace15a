/*
 * C ABI of the GB300 path tracer (include/lambda_gpu.h): context, scene compilation and upload,
 * render entry points.
 *
 * lgpu_scene_commit is the GPU counterpart of Scene::AddObject + Scene::Commit +
 * LightSampler::Commit (src/core/Scene.cpp:18-26, 114-121; src/lighting/ManyLightSampler.cpp:37-44):
 *   - every plain mesh object goes into one world BLAS (world-space triangles, object id per
 *     triangle); every mesh used through instances gets one BLAS in object space (InstanceProxy);
 *     a TLAS over instance records (world BLAS + each Instance with its world->object affine)
 *     exists only when the scene has instances;
 *   - materials and light emission sockets are compiled to bytecode;
 *   - lights become a flat table plus triangle-area CDFs, a power CDF and the light tree.
 * All buffers are copied into device memory; no caller pointer is kept.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lambda_gpu.h"
#include "lgpu_build.h"
#include "lgpu_device.cuh"
#include "lgpu_launch.h"
#include "lgpu_lighttree.h"
#include "lgpu_wavefront.cuh"

using namespace lg;

struct lgpu_context {
    int device = 0;
    int bvh_builder = LGPU_BVH_BUILD_HOST;   /* lgpu_set_bvh_builder */
    double bvh_build_ms = 0;                 /* device time of the last commit's BVH builds */
    std::string err;
    std::vector<void *> scene_allocs;
    DeviceScene S;
    bool have_scene = false;
    lgpu_stats stats;
    std::vector<int> tex_off, tex_w, tex_h;   /* image textures of the committed scene */
    std::vector<int> mask_cond, mask_marg;    /* masked-aperture distributions per texture (-1: none) */
    std::vector<float> mask_int;
    int num_media = 0, num_materials = 0;
    bool tuned = false;         /* lgpu_autotune result, used by kernel_mode AUTO */
    lgpu_tuning tuning;
    unsigned long long *d_counters = nullptr;
    int *d_err = nullptr;   /* device error word (DeviceScene::err) */
    float4 *d_film = nullptr;
    size_t film_px = 0;
    float4 *d_paths = nullptr;
    size_t paths_cap = 0;
    uint64_t *d_ids = nullptr;
    size_t ids_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    /* wavefront pool */
    void *w_states = nullptr;
    void *w_cold = nullptr;
    size_t w_state_bytes = 0;
    size_t w_slots = 0;
    float4 *w_qo = nullptr, *w_qd = nullptr, *w_res = nullptr, *w_trout = nullptr;
    int *w_resobj = nullptr, *w_qa = nullptr, *w_qb = nullptr, *w_counts = nullptr, *w_free = nullptr;
    unsigned long long *w_next = nullptr;
    int *h_count = nullptr;   /* pinned */
    cudaEvent_t w_ev[LG_NSEG + 3] = {};
    DView *d_views = nullptr;   /* view table of a batched render */
    cudaStream_t graph_stream = nullptr;   /* graph-mode work when the caller passes the default stream */
    size_t views_cap = 0;
    float4 *w_paths = nullptr;
    size_t w_paths_cap = 0;
    int last_iterations = 0;
};

namespace {

int fail(lgpu_context *c, int code, const std::string &msg);
/* Read (and clear) the device error word after the work of a render has completed on `st`. */
int check_device_error(lgpu_context *c, cudaStream_t st) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(c, LGPU_ERR_CUDA, std::string("device error word: ") + cudaGetErrorString(e));
    if (!h) return LGPU_OK;
    cudaMemsetAsync(c->d_err, 0, sizeof(int), st);
    cudaStreamSynchronize(st);
    if (h & 1) return fail(c, LGPU_ERR_QUEUE_OVERFLOW, "BVH traversal stack overflow on the device");
    return fail(c, LGPU_ERR_TIMEOUT, "path-state copy to shared memory did not complete");
}

int fail(lgpu_context *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(lgpu_context *c, cudaError_t e, const char *what) {
    return fail(c, e == cudaErrorMemoryAllocation ? LGPU_ERR_OOM : LGPU_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

void free_scene(lgpu_context *c) {
    for (void *p : c->scene_allocs) cudaFree(p);
    c->scene_allocs.clear();
    c->have_scene = false;
    std::memset(&c->S, 0, sizeof(c->S));
}

template <class T>
bool upload(lgpu_context *c, const std::vector<T> &v, const T **dst, size_t &bytes) {
    *dst = nullptr;
    if (v.empty()) return true;
    void *p = nullptr;
    const size_t sz = v.size() * sizeof(T);
    cudaError_t e = cudaMalloc(&p, sz);
    if (e != cudaSuccess) { cuda_fail(c, e, "cudaMalloc"); return false; }
    c->scene_allocs.push_back(p);
    e = cudaMemcpy(p, v.data(), sz, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cuda_fail(c, e, "cudaMemcpy"); return false; }
    *dst = reinterpret_cast<const T *>(p);
    bytes += sz;
    return true;
}

void inverse3(const float *m, float *inv) {   /* column-major 3x3 inverse in double */
    const double a = m[0], b = m[3], cc = m[6], d = m[1], e = m[4], f = m[7], g = m[2], h = m[5], i = m[8];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double det = a * A + b * B + cc * C;
    const double id = 1.0 / det;
    const double r[9] = {A * id, -(b * i - cc * h) * id, (b * f - cc * e) * id,
                         B * id, (a * i - cc * g) * id, -(a * f - cc * d) * id,
                         C * id, -(a * h - b * g) * id, (a * e - b * d) * id};
    inv[0] = (float)r[0]; inv[3] = (float)r[1]; inv[6] = (float)r[2];
    inv[1] = (float)r[3]; inv[4] = (float)r[4]; inv[7] = (float)r[5];
    inv[2] = (float)r[6]; inv[5] = (float)r[7]; inv[8] = (float)r[8];
}

inline lt::V3f v3(const float *p) { lt::V3f r; r.x = p[0]; r.y = p[1]; r.z = p[2]; return r; }

/* Host-side image of the device scene: compile_scene fills it without touching the GPU,
 * validate_scene checks every index a kernel will follow, lgpu_scene_commit uploads it. */
struct HostScene {
    DeviceScene S;
    std::vector<int> texOff, texW, texH;   /* image textures in the texel pool */
    std::vector<int> maskCond, maskMarg;   /* per texture: masked-aperture Piecewise2D offsets in fpool (-1: none) */
    std::vector<float> maskInt;
    std::vector<BvhNode> nodes;
    int bvh_depth = 0;                     /* node levels of the deepest TLAS + BLAS descent */
    mutable int bvh_stack = 0;             /* worst-case traversal stack entries (set by validate_scene) */
    std::vector<DTri> tris;
    std::vector<DInst> insts;
    std::vector<DObject> objects;
    std::vector<DMesh> meshes;
    std::vector<float4> pos, nrm, tan;
    std::vector<float2> uv;
    std::vector<uint4> tri_idx;
    std::vector<DMaterial> mats;
    std::vector<DIns> code;
    std::vector<DLight> lights;
    std::vector<DLNode> lnodes;
    std::vector<int2> treeLights, treeSlot;
    std::vector<int> lightSlot;
    std::vector<float> fpool;
    std::vector<float4> envTex;
    std::vector<DMedium> media;
};

int compile_scene(lgpu_context *c, const lgpu_scene_desc *d, HostScene &H);

bool check_ref(const HostScene &H, int ref, bool tlas, std::string &why) {
    const int idx = ref >> 4, cnt = ref & 15;
    if (idx < 0) { why = "negative child ref"; return false; }
    if (cnt == 0) { if ((size_t)idx >= H.nodes.size()) { why = "node ref out of range"; return false; } return true; }
    const size_t lim = tlas ? H.insts.size() : H.tris.size();
    if ((size_t)idx + cnt > lim) { why = tlas ? "instance leaf out of range" : "triangle leaf out of range"; return false; }
    return true;
}

/* Walk a BVH (the TLAS, or a BLAS) from its root and check refs and leaf ranges.  `need` receives
 * the most traversal-stack entries a ray can hold in it, counted the way traverse_t pushes: each
 * entry carries the entries left below it once it is popped (0 for the root), an inner node
 * pushes up to all its children, a TLAS leaf pushes the instance marker and the BLAS root.  BLAS
 * results are memoised by root since instances share them. */
bool check_bvh(const HostScene &H, int root, bool tlas, std::string &why, int &need,
               std::map<int, int> &blas_need) {
    std::vector<std::pair<int, int>> st;   /* (ref, entries below it once popped) */
    st.push_back({root, 0});
    need = 1;
    size_t visits = 0;
    while (!st.empty()) {
        auto e = st.back();
        st.pop_back();
        if (++visits > 16 * (H.nodes.size() + H.tris.size() + H.insts.size() + 4)) { why = "BVH has a cycle"; return false; }
        if (!check_ref(H, e.first, tlas, why)) return false;
        if (e.second > LGPU_STACK) { why = "BVH deeper than the traversal stack"; return false; }
        const int idx = e.first >> 4, cnt = e.first & 15;
        if (cnt == 0) {
            int ch[8], nch = 0;
#if LGPU_BVH_WIDE
            const DWide &n = H.nodes[idx];
            if (n.nchild > 8) { why = "wide node with more than eight children"; return false; }
            for (int k = 0; k < n.nchild; ++k) {
                const int m = n.meta[k], c = m & 7, off = m >> 3;
                ch[nch++] = c ? (((n.leaf_base + off) << 4) | c) : ((n.child_base + off) << 4);
            }
#else
            const DNode &n = H.nodes[idx];
            ch[nch++] = n.ch.x;
            ch[nch++] = n.ch.y;
#endif
            need = std::max(need, e.second + nch);
            for (int k = 0; k < nch; ++k) st.push_back({ch[k], e.second + nch - 1});
        } else if (tlas) {
            if (cnt != 1) { why = "TLAS leaf with more than one instance"; return false; }
            const DInst &I = H.insts[idx];
            if (I.object >= (int)H.objects.size()) { why = "instance object out of range"; return false; }
            auto it = blas_need.find(I.root);
            if (it == blas_need.end()) {
                int bn = 0;
                if (!check_bvh(H, I.root, false, why, bn, blas_need)) return false;
                it = blas_need.emplace(I.root, bn).first;
            }
            need = std::max(need, std::max(e.second + 2, e.second + 1 + it->second));
        } else {
            for (int k = 0; k < cnt; ++k) {
                const DTri &T = H.tris[idx + k];
                int prim, obj;
                std::memcpy(&prim, &T.v0.w, 4);
                std::memcpy(&obj, &T.e1.w, 4);
                if (obj >= (int)H.objects.size()) { why = "triangle object out of range"; return false; }
                if (prim < 0) { why = "negative primitive id"; return false; }
            }
        }
    }
    return true;
}

bool check_prog(const HostScene &H, int off, int len, std::string &why) {
    if (off < 0 || len < 0 || (size_t)off + len > H.code.size()) { why = "program range"; return false; }
    for (int i = 0; i < len; ++i) {
        const DIns &in = H.code[off + i];
        if (in.op >= OP_COUNT) { why = "bad opcode"; return false; }
        if (in.dst >= LGPU_MAX_REGS || in.a >= LGPU_MAX_REGS || in.b >= LGPU_MAX_REGS || in.c >= LGPU_MAX_REGS) { why = "register index"; return false; }
        if (in.op == OP_MERGE && in.sub != 255 && in.sub >= LGPU_MAX_REGS) { why = "merge register"; return false; }
        if (in.op == OP_IMAGE) {
            const int off = float_to_bits(in.k[0]), w = (int)in.k[1], h = (int)in.k[2];
            if (off < 0 || w <= 0 || h <= 0 || (size_t)off + (size_t)w * h > H.envTex.size()) { why = "image texture range"; return false; }
        }
    }
    return true;
}

bool validate_scene(const HostScene &H, std::string &why) {
    const DeviceScene &S = H.S;
    std::map<int, int> blas_need;
    if (!check_bvh(H, S.root, S.use_tlas != 0, why, H.bvh_stack, blas_need)) return false;
    if (H.bvh_stack > LGPU_STACK) {
        why = "BVH needs " + std::to_string(H.bvh_stack) + " traversal-stack entries, the device holds " + std::to_string(LGPU_STACK);
        return false;
    }
    const size_t fp = H.fpool.size();
    for (size_t t = 0; t < H.maskCond.size(); ++t) {   /* masked-aperture distributions */
        if (H.maskCond[t] < 0) continue;
        const size_t w = (size_t)H.texW[t], h = (size_t)H.texH[t];
        if ((size_t)H.maskCond[t] + h * (2 * w + 2) > fp || H.maskMarg[t] < 0 || (size_t)H.maskMarg[t] + 2 * h + 1 > fp) {
            why = "aperture mask distribution"; return false;
        }
    }
    for (size_t i = 0; i < H.objects.size(); ++i) {
        const DObject &o = H.objects[i];
        if (o.mesh < 0 || (size_t)o.mesh >= H.meshes.size() || o.material < 0 || (size_t)o.material >= H.mats.size()) { why = "object refs"; return false; }
    }
    for (size_t i = 0; i < H.meshes.size(); ++i) {
        const DMesh &m = H.meshes[i];
        if ((size_t)m.tri_off + m.num_tris > H.tri_idx.size()) { why = "mesh triangle range"; return false; }
        const size_t nv = (i + 1 < H.meshes.size() ? (size_t)H.meshes[i + 1].vtx_off : H.pos.size()) - m.vtx_off;
        for (int t = 0; t < m.num_tris; ++t) {
            const uint4 ti = H.tri_idx[m.tri_off + t];
            if (ti.x >= nv || ti.y >= nv || ti.z >= nv) { why = "vertex index"; return false; }
        }
    }
    if (H.nrm.size() != H.pos.size() || H.tan.size() != H.pos.size() || H.uv.size() != H.pos.size()) { why = "attribute sizes"; return false; }
    for (const DMaterial &m : H.mats) {
        if (m.light >= (int)H.lights.size() || m.medium_interior >= (int)H.media.size() || m.medium_exterior >= (int)H.media.size()) { why = "material refs"; return false; }
        if (!m.has_bsdf) continue;
        if (!check_prog(H, m.prog_off, m.prog_len, why)) return false;
        if (m.num_leaves < 1 || m.num_leaves > LGPU_MAX_LEAVES || m.num_tree < 1 || m.num_tree > 2 * LGPU_MAX_LEAVES - 1) { why = "bsdf tree size"; return false; }
        for (int k = 0; k < m.num_leaves; ++k)
            if (m.leaves[k].albedo >= LGPU_MAX_REGS || m.leaves[k].rough >= LGPU_MAX_REGS) { why = "leaf register"; return false; }
        for (int k = 0; k < m.num_tree; ++k) {
            const DBsdfNode &n = m.tree[k];
            if (n.kind == 0 && n.a >= m.num_leaves) { why = "bsdf leaf ref"; return false; }
            if (n.kind == 1 && (n.a >= m.num_tree || n.b >= m.num_tree || n.ratio >= LGPU_MAX_REGS)) { why = "bsdf mix ref"; return false; }
        }
    }
    const int ntl = (int)H.treeSlot.size();
    for (const DLight &L : H.lights) {
        if (L.type != LT_ENV) {
            if (!check_prog(H, L.prog_off, L.prog_len, why)) return false;
            if (L.out_reg < 0 || L.out_reg + 1 >= LGPU_MAX_REGS) { why = "emission register"; return false; }
        }
        if (L.type == LT_MESH) {
            if (L.object < 0 || (size_t)L.object >= H.objects.size()) { why = "mesh light object"; return false; }
            if (L.dist_off < 0 || (size_t)L.dist_off + 2 * L.num_tris + 1 > fp) { why = "mesh light cdf"; return false; }
            if (S.light_strategy == LGPU_LIGHT_STRATEGY_TREE && (L.tri_base < 0 || L.tri_base + L.num_tris > ntl)) { why = "mesh light tree base"; return false; }
        }
    }
    if ((size_t)S.power_cdf_off + 2 * H.lights.size() + 1 > fp) { why = "power cdf"; return false; }
    if (S.light_strategy == LGPU_LIGHT_STRATEGY_TREE && !H.lnodes.empty()) {
        if (S.tree_root != 1 || H.lnodes.size() < 2) { why = "tree root"; return false; }
        for (size_t k = 1; k < H.lnodes.size(); ++k) {
            const DLNode &n = H.lnodes[k];
            if (n.child0 == 0 || n.child0 + 1 >= (int)H.lnodes.size() || n.parent == 0 || n.parent >= (int)H.lnodes.size()) { why = "tree links"; return false; }
            if (n.child0 > 0 && (n.child0 & 1)) { why = "tree sibling pair alignment"; return false; }
            if (n.child0 > 0 && (H.lnodes[n.child0].parent != (int)k || H.lnodes[n.child0 + 1].parent != (int)k)) {
                why = "tree parent links";   /* the pdf walk climbs by parent and reads the sibling at index ^ 1 */
                return false;
            }
            if (n.first < 0 || n.num < 1 || n.first + n.num > (int)H.treeLights.size()) { why = "tree light range"; return false; }
            if (n.child0 < 0 && (n.dist_off < 0 || (size_t)n.dist_off + 2 * n.num + 1 > fp)) { why = "tree leaf cdf"; return false; }
        }
        for (const int2 &t : H.treeLights)
            if (t.x < 0 || (size_t)t.x >= H.lights.size() || t.y >= H.lights[t.x].num_tris + (H.lights[t.x].type == LT_MESH ? 0 : 1)) { why = "tree light ref"; return false; }
        for (const int2 &t : H.treeSlot)
            if (t.x < 0 || (size_t)t.x >= H.lnodes.size() || t.y < 0 || t.y >= H.lnodes[t.x].num) { why = "tree slot"; return false; }
        for (size_t i = 0; i < H.lightSlot.size(); ++i) {
            const int ls = H.lightSlot[i];
            const int ty = H.lights[i].type;
            if ((ty == LT_POINT || ty == LT_SPOT) && (ls < 0 || ls >= ntl)) { why = "light slot"; return false; }
        }
    }
    if (S.env_light >= 0) {
        const DEnv &E = S.env;
        if ((size_t)E.tex_off + (size_t)E.w * E.h > H.envTex.size()) { why = "env texture"; return false; }
        if ((size_t)E.cond_off + (size_t)E.h * (2 * E.w + 2) > fp || (size_t)E.marg_off + 2 * E.h + 1 > fp) { why = "env cdf"; return false; }
    }
    return true;
}

}  // namespace

extern "C" {

LGPU_API const char *lgpu_version(void) { return "lambda-gb300 0.3 (sm_103a, BVH2, wavefront + megakernel)"; }

LGPU_API int lgpu_set_bvh_builder(lgpu_context *c, int32_t builder) {
    if (!c) return LGPU_ERR_INVALID_ARG;
    if (builder != LGPU_BVH_BUILD_HOST && builder != LGPU_BVH_BUILD_DEVICE) return fail(c, LGPU_ERR_INVALID_ARG, "unknown BVH builder");
#if LGPU_BVH_WIDE
    if (builder == LGPU_BVH_BUILD_DEVICE) return fail(c, LGPU_ERR_INVALID_ARG, "the device builder writes binary nodes; this build uses 8-wide nodes");
#endif
    c->bvh_builder = builder;
    return LGPU_OK;
}

LGPU_API int lgpu_probe_bandwidth(lgpu_context *c, uint64_t bytes, int32_t reps, double *gbs) {
    if (!c || !gbs || reps <= 0) return LGPU_ERR_INVALID_ARG;
    const uint64_t n4 = bytes / 16;
    if (n4 < 1024) return fail(c, LGPU_ERR_INVALID_ARG, "probe buffer below 16 KiB");
    cudaError_t e = cudaSetDevice(c->device);
    float4 *buf = nullptr;
    float *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = cudaMalloc(&buf, n4 * 16);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(buf, 0, n4 * 16);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int blocks = sms * 8;   /* 8 resident 256-thread blocks per SM */
    if (e == cudaSuccess) e = read_probe(buf, n4, 1, sink, blocks, 0);   /* warm-up pass */
    if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
    if (e == cudaSuccess) e = read_probe(buf, n4, reps, sink, blocks, 0);   /* all passes in one launch */
    if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_fail(c, e, "bandwidth probe");
    *gbs = ms > 0.f ? (double)n4 * 16.0 * reps / (ms * 1e6) : 0.0;
    return LGPU_OK;
}

LGPU_API int lgpu_create(lgpu_context **out, int device) {
    if (!out) return LGPU_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return LGPU_ERR_CUDA;
    if (device < 0 || device >= n) return LGPU_ERR_INVALID_ARG;
    lgpu_context *c = new lgpu_context();
    c->device = device;
    std::memset(&c->stats, 0, sizeof(c->stats));
    std::memset(&c->S, 0, sizeof(c->S));
    e = cudaSetDevice(device);
    /* traversal counters (4) and, in the state-clock diagnostic build, cycles per program point (32) */
    if (e == cudaSuccess) e = cudaMalloc(&c->d_counters, 36 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(c->d_counters, 0, 36 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e != cudaSuccess) { delete c; return LGPU_ERR_CUDA; }
    *out = c;
    return LGPU_OK;
}

LGPU_API void lgpu_destroy(lgpu_context *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    free_scene(c);
    cudaFree(c->d_counters);
    cudaFree(c->d_err);
    cudaFree(c->d_film);
    cudaFree(c->d_paths);
    cudaFree(c->d_ids);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (auto &x : c->w_ev) if (x) cudaEventDestroy(x);
    cudaFree(c->d_views);
    if (c->graph_stream) cudaStreamDestroy(c->graph_stream);
    cudaFree(c->w_states); cudaFree(c->w_cold); cudaFree(c->w_qo); cudaFree(c->w_qd); cudaFree(c->w_res); cudaFree(c->w_resobj);
    cudaFree(c->w_trout);
    cudaFree(c->w_qa); cudaFree(c->w_qb); cudaFree(c->w_counts); cudaFree(c->w_next); cudaFree(c->w_paths); cudaFree(c->w_free);
    if (c->h_count) cudaFreeHost(c->h_count);
    delete c;
}

LGPU_API const char *lgpu_last_error(const lgpu_context *c) { return c ? c->err.c_str() : "null context"; }

/* Compile and validate a scene on the host only (no CUDA call); writes a short report. */
LGPU_API int lgpu_scene_check(const lgpu_scene_desc *d, char *report, size_t report_size) {
    lgpu_context tmp;
    HostScene H;
    int rc = compile_scene(&tmp, d, H);
    std::string msg;
    if (rc == LGPU_OK) {
        std::string why;
        if (!validate_scene(H, why)) { rc = LGPU_ERR_INVALID_SCENE; msg = "validation: " + why; }
        else {
            msg = "ok nodes=" + std::to_string(H.nodes.size()) + " depth=" + std::to_string(H.bvh_depth) +
                  " stack=" + std::to_string(H.bvh_stack) +
                  " tris=" + std::to_string(H.tris.size()) +
                  " insts=" + std::to_string(H.insts.size()) + " prog=" + std::to_string(H.code.size()) +
                  " lnodes=" + std::to_string(H.lnodes.size()) + " fpool=" + std::to_string(H.fpool.size()) +
                  " tree_power=" + std::to_string(H.S.tree_power);
        }
    } else msg = tmp.err;
    if (report && report_size) {
        std::strncpy(report, msg.c_str(), report_size - 1);
        report[report_size - 1] = 0;
    }
    return rc;
}

LGPU_API int lgpu_get_stats(const lgpu_context *c, lgpu_stats *out) {
    if (!c || !out) return LGPU_ERR_INVALID_ARG;
    *out = c->stats;
    return LGPU_OK;
}

}  // extern "C"

namespace {
int compile_scene(lgpu_context *c, const lgpu_scene_desc *d, HostScene &H) {
    if (!d) return LGPU_ERR_INVALID_ARG;
    /* ---------------- validation */
    for (int i = 0; i < d->num_objects; ++i) {
        const lgpu_object_desc &o = d->objects[i];
        if (o.mesh < 0 || o.mesh >= d->num_meshes) return fail(c, LGPU_ERR_INVALID_SCENE, "object " + std::to_string(i) + " has no mesh");
        if (o.material < 0 || o.material >= d->num_materials) return fail(c, LGPU_ERR_INVALID_SCENE, "object " + std::to_string(i) + " has no material");
    }
    for (int i = 0; i < d->num_meshes; ++i) {
        const lgpu_mesh_desc &m = d->meshes[i];
        for (uint32_t t = 0; t < 3 * m.num_triangles; ++t)
            if (m.triangles[t] >= m.num_vertices) return fail(c, LGPU_ERR_INVALID_SCENE, "mesh " + std::to_string(i) + " indexes a missing vertex");
    }
    if (d->num_lights == 0) return fail(c, LGPU_ERR_INVALID_SCENE, "scene has no light (the reference requires one)");

    std::vector<float> &fpool = H.fpool;
    DeviceScene &S = H.S;
    std::memset(&S, 0, sizeof(S));
    S.has_volumes = d->has_volumes;
    S.light_strategy = d->light_strategy;
    S.num_lights = d->num_lights;

    /* ---------------- meshes: vertex attributes */
    std::vector<float4> &pos = H.pos, &nrm = H.nrm, &tan = H.tan;
    std::vector<float2> &uv = H.uv;
    std::vector<uint4> &tri_idx = H.tri_idx;
    std::vector<DMesh> &meshes = H.meshes;
    meshes.resize(d->num_meshes);
    for (int i = 0; i < d->num_meshes; ++i) {
        const lgpu_mesh_desc &m = d->meshes[i];
        DMesh &dm = meshes[i];
        dm.vtx_off = (int)pos.size();
        dm.tri_off = (int)tri_idx.size();
        dm.num_tris = (int)m.num_triangles;
        dm.flags = ((m.normals && m.tangents) ? 1 : 0) | (m.uvs ? 2 : 0);
        for (uint32_t v = 0; v < m.num_vertices; ++v) {
            pos.push_back(make_float4(m.vertices[3 * v], m.vertices[3 * v + 1], m.vertices[3 * v + 2], 0.f));
            nrm.push_back((dm.flags & 1) ? make_float4(m.normals[3 * v], m.normals[3 * v + 1], m.normals[3 * v + 2], 0.f) : make_float4(0, 0, 0, 0));
            tan.push_back((dm.flags & 1) ? make_float4(m.tangents[4 * v], m.tangents[4 * v + 1], m.tangents[4 * v + 2], m.tangents[4 * v + 3]) : make_float4(0, 0, 0, 0));
            uv.push_back(m.uvs ? make_float2(m.uvs[2 * v], m.uvs[2 * v + 1]) : make_float2(0, 0));
        }
        for (uint32_t t = 0; t < m.num_triangles; ++t)
            tri_idx.push_back(make_uint4(m.triangles[3 * t], m.triangles[3 * t + 1], m.triangles[3 * t + 2], 0u));
    }

    /* ---------------- objects */
    std::vector<DObject> &objects = H.objects;
    objects.resize(d->num_objects);
    lt::Box sceneBox;
    bool firstBox = true;
    std::vector<lt::Box> objBox(d->num_objects);
    for (int i = 0; i < d->num_objects; ++i) {
        const lgpu_object_desc &o = d->objects[i];
        DObject &ob = objects[i];
        ob.mesh = o.mesh; ob.material = o.material; ob.kind = o.kind;
        static const float id12[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
        const float *x = o.kind == 1 ? o.xfm : id12;
        for (int k = 0; k < 9; ++k) ob.m[k] = x[k];
        for (int k = 0; k < 3; ++k) ob.t[k] = x[9 + k];
        ob.identity = 1;
        for (int k = 0; k < 12; ++k) if (x[k] != id12[k]) ob.identity = 0;
        float inv[9];
        inverse3(ob.m, inv);
        for (int r = 0; r < 3; ++r) for (int cidx = 0; cidx < 3; ++cidx) ob.nrm[cidx * 3 + r] = inv[r * 3 + cidx];
        /* world bounds from transformed vertices, as the oracle computes them */
        const lgpu_mesh_desc &m = d->meshes[o.mesh];
        lt::Box b;
        for (uint32_t v = 0; v < m.num_vertices; ++v) {
            const float *p = m.vertices + 3 * v;
            lt::V3f w;
            if (ob.identity) w = v3(p);
            else {
                w.x = ob.m[0] * p[0] + ob.m[3] * p[1] + ob.m[6] * p[2];
                w.y = ob.m[1] * p[0] + ob.m[4] * p[1] + ob.m[7] * p[2];
                w.z = ob.m[2] * p[0] + ob.m[5] * p[1] + ob.m[8] * p[2];
                w.x = w.x + ob.t[0]; w.y = w.y + ob.t[1]; w.z = w.z + ob.t[2];
            }
            lt::Box pb; pb.mn = w; pb.mx = w;
            b = v == 0 ? pb : lt::Box::unite(b, pb);
        }
        objBox[i] = b;
        sceneBox = firstBox ? b : lt::Box::unite(sceneBox, b);
        firstBox = false;
    }

    /* ---------------- geometry: BLAS / TLAS */
    std::vector<BvhNode> &nodes = H.nodes;
    std::vector<DTri> &tris = H.tris;
    std::vector<DInst> &insts = H.insts;
    auto make_tri = [&](const lgpu_mesh_desc &m, uint32_t t, int objId) {
        const float *v0 = m.vertices + 3 * m.triangles[3 * t], *v1 = m.vertices + 3 * m.triangles[3 * t + 1], *v2 = m.vertices + 3 * m.triangles[3 * t + 2];
        DTri T;
        T.v0 = make_float4(v0[0], v0[1], v0[2], bits_to_float((int)t));
        T.e1 = make_float4(v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2], bits_to_float(objId));
        T.e2 = make_float4(v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2], 0.f);
        return T;
    };
    auto tri_box = [&](const lgpu_mesh_desc &m, uint32_t t) {
        Aabb b;
        for (int k = 0; k < 3; ++k) { b.lo[k] = INFINITY; b.hi[k] = -INFINITY; }
        for (int j = 0; j < 3; ++j) {
            const float *p = m.vertices + 3 * m.triangles[3 * t + j];
            for (int k = 0; k < 3; ++k) { b.lo[k] = std::min(b.lo[k], p[k]); b.hi[k] = std::max(b.hi[k], p[k]); }
        }
        return b;
    };
    int maxDepth = 0;
    c->bvh_build_ms = 0;
    /* one BVH: the host's binned SAH, or the device's LBVH when selected (binary layout only) */
    std::string bvh_err;
    auto bvh = [&](const std::vector<Aabb> &boxes, int max_leaf, int node_base, int prim_base, DeviceBvh &out) -> bool {
#if !LGPU_BVH_WIDE
        if (c->bvh_builder == LGPU_BVH_BUILD_DEVICE && boxes.size() >= 2) {
            BvhOut b;
            float ms = 0.f;
            if (build_lbvh_device(boxes, node_base, prim_base, b, &ms, bvh_err) != 0) return false;
            c->bvh_build_ms += ms;
            out.nodes.swap(b.nodes); out.order.swap(b.order); out.root_ref = b.root_ref; out.depth = b.max_depth;
            return true;
        }
#endif
        build_device_bvh(boxes, max_leaf, node_base, prim_base, out);
        return true;
    };
    /* world BLAS over plain mesh objects */
    std::vector<std::pair<int, uint32_t>> worldPrims;   /* (object, triangle) */
    bool anyInstance = false;
    for (int i = 0; i < d->num_objects; ++i) {
        if (d->objects[i].kind == 1) { anyInstance = true; continue; }
        const lgpu_mesh_desc &m = d->meshes[d->objects[i].mesh];
        for (uint32_t t = 0; t < m.num_triangles; ++t) worldPrims.push_back({i, t});
    }
    int worldRoot;
    {
        std::vector<Aabb> boxes(worldPrims.size());
        for (size_t k = 0; k < worldPrims.size(); ++k) boxes[k] = tri_box(d->meshes[d->objects[worldPrims[k].first].mesh], worldPrims[k].second);
        DeviceBvh bo;
        if (!bvh(boxes, 4, (int)nodes.size(), (int)tris.size(), bo)) return fail(c, LGPU_ERR_CUDA, bvh_err);
        maxDepth = std::max(maxDepth, bo.depth);
        nodes.insert(nodes.end(), bo.nodes.begin(), bo.nodes.end());
        for (uint32_t k : bo.order) {
            const auto &wp = worldPrims[k];
            tris.push_back(make_tri(d->meshes[d->objects[wp.first].mesh], wp.second, wp.first));
        }
        worldRoot = bo.root_ref;
    }
    if (anyInstance) {
        std::vector<int> blasRoot(d->num_meshes, -1);
        std::vector<Aabb> instBoxes;
        if (!worldPrims.empty()) {
            DInst I;
            I.r0 = make_float4(1, 0, 0, 0); I.r1 = make_float4(0, 1, 0, 0); I.r2 = make_float4(0, 0, 1, 0);
            I.root = worldRoot; I.object = -1; I.pad0 = I.pad1 = 0;
            insts.push_back(I);
            Aabb wb;
            for (int k = 0; k < 3; ++k) { wb.lo[k] = INFINITY; wb.hi[k] = -INFINITY; }
            for (int i = 0; i < d->num_objects; ++i) {
                if (d->objects[i].kind == 1) continue;
                const lt::Box &b = objBox[i];
                wb.lo[0] = std::min(wb.lo[0], b.mn.x); wb.lo[1] = std::min(wb.lo[1], b.mn.y); wb.lo[2] = std::min(wb.lo[2], b.mn.z);
                wb.hi[0] = std::max(wb.hi[0], b.mx.x); wb.hi[1] = std::max(wb.hi[1], b.mx.y); wb.hi[2] = std::max(wb.hi[2], b.mx.z);
            }
            instBoxes.push_back(wb);
        }
        for (int i = 0; i < d->num_objects; ++i) {
            const lgpu_object_desc &o = d->objects[i];
            if (o.kind != 1) continue;
            if (blasRoot[o.mesh] < 0) {
                const lgpu_mesh_desc &m = d->meshes[o.mesh];
                std::vector<Aabb> boxes(m.num_triangles);
                for (uint32_t t = 0; t < m.num_triangles; ++t) boxes[t] = tri_box(m, t);
                DeviceBvh bo;
                if (!bvh(boxes, 4, (int)nodes.size(), (int)tris.size(), bo)) return fail(c, LGPU_ERR_CUDA, bvh_err);
                maxDepth = std::max(maxDepth, bo.depth);
                nodes.insert(nodes.end(), bo.nodes.begin(), bo.nodes.end());
                for (uint32_t k : bo.order) tris.push_back(make_tri(m, k, -1));
                blasRoot[o.mesh] = bo.root_ref;
            }
            const DObject &ob = objects[i];
            float inv[9];
            inverse3(ob.m, inv);
            /* world -> object: x_obj = inv * (x - t); rows of inv, translation in w */
            DInst I;
            I.r0 = make_float4(inv[0], inv[3], inv[6], ob.t[0]);
            I.r1 = make_float4(inv[1], inv[4], inv[7], ob.t[1]);
            I.r2 = make_float4(inv[2], inv[5], inv[8], ob.t[2]);
            I.root = blasRoot[o.mesh]; I.object = i; I.pad0 = I.pad1 = 0;
            insts.push_back(I);
            const lt::Box &b = objBox[i];
            Aabb ab;
            ab.lo[0] = b.mn.x; ab.lo[1] = b.mn.y; ab.lo[2] = b.mn.z;
            ab.hi[0] = b.mx.x; ab.hi[1] = b.mx.y; ab.hi[2] = b.mx.z;
            instBoxes.push_back(ab);
        }
        DeviceBvh bo;
        if (!bvh(instBoxes, 1, (int)nodes.size(), 0, bo)) return fail(c, LGPU_ERR_CUDA, bvh_err);
        nodes.insert(nodes.end(), bo.nodes.begin(), bo.nodes.end());
        std::vector<DInst> reordered;
        for (uint32_t k : bo.order) reordered.push_back(insts[k]);
        insts.swap(reordered);
        S.root = bo.root_ref;
        S.use_tlas = 1;
        maxDepth += bo.depth;
    } else {
        S.root = worldRoot;
        S.use_tlas = 0;
    }
    H.bvh_depth = maxDepth;   /* the stack bound is checked by validate_scene */

    /* ---------------- materials */
    std::vector<DIns> &code = H.code;
    /* image textures first: their texels share the float4 pool of the environment map */
    std::vector<int> &texOff = H.texOff;
    for (int t = 0; t < d->num_textures; ++t) {
        const lgpu_texture_desc &td = d->textures[t];
        if (!td.rgba || td.width <= 0 || td.height <= 0) return fail(c, LGPU_ERR_INVALID_SCENE, "image texture without texels");
        texOff.push_back((int)H.envTex.size());
        H.texW.push_back(td.width);
        H.texH.push_back(td.height);
        for (int k = 0; k < td.width * td.height; ++k)
            H.envTex.push_back(make_float4(td.rgba[4 * k], td.rgba[4 * k + 1], td.rgba[4 * k + 2], td.rgba[4 * k + 3]));
        H.maskCond.push_back(-1); H.maskMarg.push_back(-1); H.maskInt.push_back(0.f);
        if (td.aperture_mask) {
            /* MaskedAperture::InitDistribution (Aperture.cpp:38-51): |red| of GetPixelUV at texel
             * corners (bilinear, Texture.h:71-81), then Piecewise2D (Piecewise.cpp:40-58) */
            const int w = td.width, h = td.height;
            std::vector<float> img((size_t)w * h);
            for (int y = 0; y < h; ++y) {
                const float vp = (float)y / (float)h;
                for (int x = 0; x < w; ++x) {
                    const float up = (float)x / (float)w;
                    const float fx = std::min((float)(w - 1), std::max(std::min(up, 1.f), 0.f) * (float)w);
                    const float fy = std::min((float)(h - 1), std::max(std::min(vp, 1.f), 0.f) * (float)h);
                    const unsigned xi = (unsigned)fx, yi = (unsigned)fy;
                    const unsigned x1 = std::min(xi + 1, (unsigned)w - 1), y1 = std::min(yi + 1, (unsigned)h - 1);
                    const float r00 = td.rgba[4 * ((size_t)yi * w + xi)], r10 = td.rgba[4 * ((size_t)yi * w + x1)];
                    const float r01 = td.rgba[4 * ((size_t)y1 * w + xi)], r11 = td.rgba[4 * ((size_t)y1 * w + x1)];
                    const float ya = r00 + (r10 - r00) * (fx - (float)xi);
                    const float yb = r01 + (r11 - r01) * (fx - (float)xi);
                    img[x + (size_t)y * w] = std::abs(ya + (yb - ya) * (fy - (float)yi));
                }
            }
            std::vector<float> rowInt(h);
            H.maskCond[t] = (int)H.fpool.size();
            for (int y = 0; y < h; ++y) {
                int off;
                rowInt[y] = lt::piecewise1d(&img[(size_t)y * w], (unsigned)w, H.fpool, off);
                H.fpool.push_back(rowInt[y]);
            }
            int marg;
            H.maskInt[t] = lt::piecewise1d(rowInt.data(), (unsigned)h, H.fpool, marg);
            H.maskMarg[t] = marg;
        }
    }
    GraphCompiler gc;
    gc.d = d;
    gc.code = &code;
    gc.tex_off = &texOff;
    std::vector<DMaterial> &mats = H.mats;
    mats.resize(d->num_materials);
    for (int i = 0; i < d->num_materials; ++i) {
        const lgpu_material_desc &md = d->materials[i];
        DMaterial &m = mats[i];
        std::memset(&m, 0, sizeof(m));
        m.light = md.light;
        m.medium_interior = md.medium_interior;
        m.medium_exterior = md.medium_exterior;
        m.has_bsdf = md.bxdf_node >= 0;
        m.prog_off = 0; m.prog_len = 0;
        if (md.light >= d->num_lights) return fail(c, LGPU_ERR_INVALID_SCENE, "material light index out of range");
        if (md.medium_interior >= d->num_media || md.medium_exterior >= d->num_media) return fail(c, LGPU_ERR_INVALID_SCENE, "material medium index out of range");
        if (m.has_bsdf && !gc.compile_material(md.bxdf_node, m))
            return fail(c, LGPU_ERR_UNSUPPORTED_NODE, "material " + std::to_string(i) + ": " + gc.err);
    }

    /* ---------------- lights */
    std::vector<DLight> &lights = H.lights;
    lights.resize(d->num_lights);
    std::vector<lt::TreeLightIn> treeIn;
    std::vector<int2> treeRef;      /* (light, tri) per tree light, input order */
    std::vector<int> &lightSlot = H.lightSlot;
    lightSlot.assign(d->num_lights, -1);
    std::vector<float> lightPower(d->num_lights, 0.f);
    int envLight = -1;
    DEnv env;
    std::memset(&env, 0, sizeof(env));
    std::vector<float4> &envTex = H.envTex;
    const float PIf = 3.14159265358979323846f;
    for (int i = 0; i < d->num_lights; ++i) {
        const lgpu_light_desc &ld = d->lights[i];
        DLight &L = lights[i];
        std::memset(&L, 0, sizeof(L));
        L.intensity = ld.intensity;
        L.object = ld.object;
        L.dist_off = -1;
        L.tri_base = -1;
        if (ld.type != LGPU_LIGHT_ENVIRONMENT) {
            if (ld.emission_node < 0 || ld.emission_node >= d->num_nodes) return fail(c, LGPU_ERR_INVALID_SCENE, "light " + std::to_string(i) + " has no emission socket");
            if (!gc.compile_emission(ld.emission_node, ld.emission_socket, L.prog_off, L.prog_len, L.out_reg))
                return fail(c, LGPU_ERR_UNSUPPORTED_NODE, "light " + std::to_string(i) + ": " + gc.err);
            L.em_folded = gc.fold_emission(L.prog_off, L.prog_len, L.out_reg, L.em) ? 1 : 0;
        }
        if (ld.type == LGPU_LIGHT_MESH) {
            if (ld.object < 0 || ld.object >= d->num_objects) return fail(c, LGPU_ERR_INVALID_SCENE, "mesh light without object");
            L.type = LT_MESH;
            const lgpu_mesh_desc &m = d->meshes[d->objects[ld.object].mesh];
            std::vector<float> areas(m.num_triangles);
            float meshArea = 0;
            L.tri_base = (int)treeIn.size();
            /* TriangleLight::Irradiance: emission luminance at 3x3 barycentric points (RGB semantics) */
            for (uint32_t t = 0; t < m.num_triangles; ++t) {
                const lt::V3f a = v3(m.vertices + 3 * m.triangles[3 * t]), b = v3(m.vertices + 3 * m.triangles[3 * t + 1]),
                              cc = v3(m.vertices + 3 * m.triangles[3 * t + 2]);
                const lt::V3f e1 = b - a, e2 = cc - a;
                const lt::V3f cr = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
                const float crm = std::sqrt(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
                areas[t] = crm * .5f;
                meshArea += crm;
                float irr = 0.f;
                const float inv3 = 1.f / 3.f;
                for (unsigned aa = 0; aa < 3; ++aa)
                    for (unsigned bb = 0; bb < 3; ++bb) {
                        ShadeCtx sc;
                        std::memset(&sc, 0, sizeof(sc));
                        sc.eta = 1.001f;
                        sc.texels = H.envTex.data();
                        if (m.uvs) {
                            const float *u0 = m.uvs + 2 * m.triangles[3 * t], *u1 = m.uvs + 2 * m.triangles[3 * t + 1], *u2 = m.uvs + 2 * m.triangles[3 * t + 2];
                            const float fu = (float)aa * inv3, fv = (float)bb * inv3;
                            sc.uv = make_float2(u0[0] + (u1[0] - u0[0]) * fu + (u2[0] - u0[0]) * fv, u0[1] + (u1[1] - u0[1]) * fu + (u2[1] - u0[1]) * fv);
                        }
                        float4 R[LGPU_MAX_REGS];
                        Lambda4 lam;
                        run_prog<3>(code.data() + L.prog_off, L.prog_len, sc, lam, R);
                        irr += spec_y<3>(Spec<3>::from4(R[L.out_reg]), lam);
                    }
                const float irradiance = irr * inv3 * inv3 * ld.intensity;
                lt::TreeLightIn tl;
                lt::Box tb; tb.mn = a; tb.mx = a;
                lt::Box pb; pb.mn = b; pb.mx = b;
                tb = lt::Box::unite(tb, pb);
                pb.mn = cc; pb.mx = cc;
                tb = lt::Box::unite(tb, pb);
                tl.b = tb;
                const float inv2a = (float)(areas[t] * 2.);
                tl.dir = {cr.x / inv2a, cr.y / inv2a, cr.z / inv2a};
                tl.dir = lt::V3f{cr.x * (1.f / inv2a), cr.y * (1.f / inv2a), cr.z * (1.f / inv2a)};
                tl.power = irradiance * areas[t];
                treeIn.push_back(tl);
                treeRef.push_back(make_int2(i, (int)t));
            }
            L.num_tris = (int)m.num_triangles;
            L.integral = lt::piecewise1d(areas.data(), m.num_triangles, fpool, L.dist_off);
            L.power = ld.intensity * (meshArea * .5f);
        } else if (ld.type == LGPU_LIGHT_POINT || ld.type == LGPU_LIGHT_SPOT) {
            L.type = ld.type == LGPU_LIGHT_POINT ? LT_POINT : LT_SPOT;
            L.pos = make_float3(ld.position[0], ld.position[1], ld.position[2]);
            L.axis = make_float3(ld.axis[0], ld.axis[1], ld.axis[2]);
            L.cosCone = std::cos(ld.cone_angle);
            L.cosFall = std::cos(ld.falloff_start);
            L.power = L.type == LT_POINT ? ld.intensity * (4 * PIf)
                                         : ld.intensity * (2.f * PIf - (1 - .5f * (L.cosFall + L.cosCone)));
        } else if (ld.type == LGPU_LIGHT_ENVIRONMENT) {
            if (envLight >= 0) return fail(c, LGPU_ERR_INVALID_SCENE, "more than one environment light");
            if (!ld.env_texture || ld.env_width <= 0 || ld.env_height <= 0) return fail(c, LGPU_ERR_INVALID_SCENE, "environment light without texture");
            L.type = LT_ENV;
            envLight = i;
            const int w = ld.env_width, h = ld.env_height;
            env.w = w; env.h = h; env.present = 1; env.intensity = ld.intensity;
            env.offx = ld.offset[0]; env.offy = ld.offset[1];
            env.tex_off = (int)envTex.size();
            for (int k = 0; k < w * h; ++k) envTex.push_back(make_float4(ld.env_texture[3 * k], ld.env_texture[3 * k + 1], ld.env_texture[3 * k + 2], 0.f));
            /* EnvironmentLight constructor (EnvironmentLight.cpp:9-22): luminance * sin(theta) */
            std::vector<float> img((size_t)w * h);
            for (int y = 0; y < h; ++y) {
                const float vp = (float)y / (float)h;
                const float sinT = std::sin(PIf * float(y + .5) / float(h));
                for (int x = 0; x < w; ++x) {
                    const float up = (float)x / (float)w;
                    /* bilinear fetch at a texel corner = that texel */
                    const float fx = std::min((float)(w - 1), std::max(std::min(up, 1.f), 0.f) * (float)w);
                    const float fy = std::min((float)(h - 1), std::max(std::min(vp, 1.f), 0.f) * (float)h);
                    const unsigned xi = (unsigned)fx, yi = (unsigned)fy;
                    const unsigned x1 = std::min(xi + 1, (unsigned)w - 1), y1 = std::min(yi + 1, (unsigned)h - 1);
                    const float *t00 = ld.env_texture + 3 * ((size_t)yi * w + xi), *t10 = ld.env_texture + 3 * ((size_t)yi * w + x1);
                    const float *t01 = ld.env_texture + 3 * ((size_t)y1 * w + xi), *t11 = ld.env_texture + 3 * ((size_t)y1 * w + x1);
                    float rgb[3];
                    for (int k = 0; k < 3; ++k) {
                        const float ya = t00[k] + (t10[k] - t00[k]) * (fx - (float)xi);
                        const float yb = t01[k] + (t11[k] - t01[k]) * (fx - (float)xi);
                        rgb[k] = ya + (yb - ya) * (fy - (float)yi);
                    }
                    const float lum = 0.212671f * rgb[0] + 0.715160f * rgb[1] + 0.072169f * rgb[2];
                    img[x + (size_t)y * w] = std::abs(lum) * sinT;
                }
            }
            /* Piecewise2D: per row CDF (w+1) + func (w) + integral (1); marginal CDF + func */
            std::vector<float> rowInt(h);
            env.cond_off = (int)fpool.size();
            for (int y = 0; y < h; ++y) {
                int off;
                rowInt[y] = lt::piecewise1d(&img[(size_t)y * w], (unsigned)w, fpool, off);
                fpool.push_back(rowInt[y]);
            }
            env.marg_integral = lt::piecewise1d(rowInt.data(), (unsigned)h, fpool, env.marg_off);
            const float radius = std::max(std::max(sceneBox.mx.x - sceneBox.mn.x, sceneBox.mx.y - sceneBox.mn.y), sceneBox.mx.z - sceneBox.mn.z);
            L.power = ld.intensity * (PIf * radius * radius);
        } else {
            return fail(c, LGPU_ERR_INVALID_SCENE, "unknown light type");
        }
        lightPower[i] = L.power;
        if (L.type == LT_POINT || L.type == LT_SPOT) {
            lt::TreeLightIn tl;
            tl.b.mn = v3(ld.position); tl.b.mx = tl.b.mn;
            tl.dir = L.type == LT_POINT ? lt::V3f{0, 1, 0} : v3(ld.axis);
            tl.power = L.power;
            treeIn.push_back(tl);
            treeRef.push_back(make_int2(i, -1));
        }
    }
    S.env = env;
    S.env_light = envLight;
    /* tree lights: triangle lights first (input order), then point / spot lights (ManyLightSampler::InitLights) */
    {
        std::vector<lt::TreeLightIn> ordered;
        std::vector<int2> orderedRef;
        for (size_t k = 0; k < treeIn.size(); ++k) if (treeRef[k].y >= 0) { ordered.push_back(treeIn[k]); orderedRef.push_back(treeRef[k]); }
        for (size_t k = 0; k < treeIn.size(); ++k) if (treeRef[k].y < 0) { ordered.push_back(treeIn[k]); orderedRef.push_back(treeRef[k]); }
        treeIn.swap(ordered);
        treeRef.swap(orderedRef);
        int base = 0;
        for (int i = 0; i < d->num_lights; ++i)
            if (lights[i].type == LT_MESH) { lights[i].tri_base = base; base += lights[i].num_tris; }
    }
    /* power sampler CDF (PowerLightSampler::Commit, LightSampler.cpp:25-35) */
    {
        float tot = 0;
        for (int i = 0; i < d->num_lights; ++i) tot += lightPower[i];
        S.power_integral = lt::piecewise1d(lightPower.data(), (unsigned)d->num_lights, fpool, S.power_cdf_off);
        S.inv_total_power = 1.f / tot;
    }
    std::vector<int2> &treeLights = H.treeLights, &treeSlot = H.treeSlot;
    std::vector<DLNode> &lnodes = H.lnodes;
    if (d->light_strategy == LGPU_LIGHT_STRATEGY_TREE) {
        lt::TreeOut to;
        lt::build_light_tree(treeIn, fpool, to);
        lnodes = to.nodes;
        S.tree_root = to.root;
        S.tree_power = to.tree_power;
        S.inf_power = envLight >= 0 ? lightPower[envLight] * .1f : 0.f;
        S.num_tree_lights = (int)treeIn.size();
        treeLights.resize(to.order.size());
        for (size_t k = 0; k < to.order.size(); ++k) treeLights[k] = treeRef[to.order[k]];
        /* input index -> (leaf, slot) */
        std::vector<int2> slotOfInput(treeIn.size(), make_int2(-1, -1));
        for (size_t ni = 0; ni < lnodes.size(); ++ni) {
            const DLNode &n = lnodes[ni];
            if (ni == 0 || n.child0 >= 0) continue;
            for (int k = 0; k < n.num; ++k) slotOfInput[to.order[n.first + k]] = make_int2((int)ni, k);
        }
        /* tree_slot is indexed by: mesh lights -> tri_base + tri, other lights -> their slot index */
        treeSlot.resize(treeIn.size());
        for (size_t k = 0; k < treeIn.size(); ++k) {
            const int2 r = treeRef[k];
            if (r.y >= 0) treeSlot[lights[r.x].tri_base + r.y] = slotOfInput[k];
            else { lightSlot[r.x] = (int)k; treeSlot[k] = slotOfInput[k]; }
        }
        if (treeIn.empty() && envLight < 0) return fail(c, LGPU_ERR_INVALID_SCENE, "light tree is empty");
        if (!treeIn.empty() && to.root < 0)
            return fail(c, LGPU_ERR_INVALID_SCENE, to.root == -2 ? "light-tree cone with an emission angle other than pi/2"
                                                                 : "light tree builder produced unpaired children");
    }

    /* ---------------- media */
    std::vector<DMedium> &media = H.media;
    media.resize(d->num_media);
    for (int i = 0; i < d->num_media; ++i) {
        DMedium &m = media[i];
        std::memset(&m, 0, sizeof(m));
        for (int k = 0; k < 3; ++k) { m.sa[k] = d->media[i].sigma_a[k]; m.ss[k] = d->media[i].sigma_s[k]; }
        m.g = d->media[i].g;
    }

    return LGPU_OK;
}
}  // namespace

extern "C" {

LGPU_API int lgpu_scene_commit(lgpu_context *c, const lgpu_scene_desc *d) {
    if (!c || !d) return LGPU_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    free_scene(c);
    HostScene H;
    int rc = compile_scene(c, d, H);
    if (rc) return rc;
    std::string why;
    if (!validate_scene(H, why)) return fail(c, LGPU_ERR_INVALID_SCENE, "compiled scene failed validation: " + why);
    DeviceScene S = H.S;
    size_t bytes = 0;
    const auto &nodes = H.nodes; const auto &tris = H.tris; const auto &insts = H.insts; const auto &objects = H.objects;
    const auto &meshes = H.meshes; const auto &pos = H.pos; const auto &nrm = H.nrm; const auto &tan = H.tan;
    const auto &uv = H.uv; const auto &tri_idx = H.tri_idx; const auto &mats = H.mats; const auto &code = H.code;
    const auto &lights = H.lights; const auto &lnodes = H.lnodes; const auto &treeLights = H.treeLights;
    const auto &treeSlot = H.treeSlot; const auto &lightSlot = H.lightSlot; const auto &fpool = H.fpool;
    const auto &envTex = H.envTex; const auto &media = H.media;
    /* ---------------- upload */
    bool ok = upload(c, nodes, &S.nodes, bytes) && upload(c, tris, &S.tris, bytes) && upload(c, insts, &S.insts, bytes) &&
              upload(c, objects, &S.objects, bytes) && upload(c, meshes, &S.meshes, bytes) && upload(c, pos, &S.pos, bytes) &&
              upload(c, nrm, &S.nrm, bytes) && upload(c, tan, &S.tan, bytes) && upload(c, uv, &S.uv, bytes) &&
              upload(c, tri_idx, &S.tri_idx, bytes) && upload(c, mats, &S.materials, bytes) && upload(c, code, &S.prog, bytes) &&
              upload(c, lights, &S.lights, bytes) && upload(c, lnodes, &S.lnodes, bytes) &&
              upload(c, treeLights, &S.tree_lights, bytes) && upload(c, treeSlot, &S.tree_slot, bytes) &&
              upload(c, lightSlot, &S.light_slot, bytes) && upload(c, fpool, &S.fpool, bytes) &&
              upload(c, envTex, &S.env_tex, bytes) && upload(c, media, &S.media, bytes);
    if (!ok) { free_scene(c); return c->err.find("alloc") != std::string::npos ? LGPU_ERR_OOM : LGPU_ERR_CUDA; }
    S.err = c->d_err;
    c->S = S;
    c->tex_off = H.texOff; c->tex_w = H.texW; c->tex_h = H.texH;
    c->mask_cond = H.maskCond; c->mask_marg = H.maskMarg; c->mask_int = H.maskInt;
    c->num_media = (int)H.media.size();
    c->num_materials = (int)H.mats.size();
    c->have_scene = true;
    c->stats.bvh_nodes = nodes.size();
    c->stats.bvh_build_ms = c->bvh_build_ms;
    c->stats.bvh_bytes = nodes.size() * sizeof(BvhNode);
    c->stats.tri_bytes = tris.size() * sizeof(DTri);
    c->stats.node_bytes = sizeof(BvhNode);
    c->stats.tri_record_bytes = sizeof(DTri);
    c->stats.device_bytes = bytes;
    return LGPU_OK;
}

}  // extern "C"

namespace {

CamParams make_cam(const lgpu_context *c, const lgpu_camera_desc *cd, const lgpu_render_opts *o) {
    CamParams cam;
    std::memset(&cam, 0, sizeof(cam));
    cam.o = make_float3(cd->origin[0], cd->origin[1], cd->origin[2]);
    cam.x = make_float3(cd->x_hat[0], cd->x_hat[1], cd->x_hat[2]);
    cam.y = make_float3(cd->y_hat[0], cd->y_hat[1], cd->y_hat[2]);
    cam.z = make_float3(cd->z_hat[0], cd->z_hat[1], cd->z_hat[2]);
    cam.tanFov = (float)std::tan(.5 * cd->fov);   /* Camera::SetFov (Camera.cpp:34-37) */
    cam.tanFov2 = 2 * cam.tanFov;
    cam.aspect = (float)o->height / (float)o->width;
    cam.xi = 1.f / (float)o->width;
    cam.yi = 1.f / (float)o->height;
    cam.W = o->width;
    cam.H = o->height;
    cam.type = cd->type;
    cam.aperture = cd->type == LGPU_CAMERA_THIN_LENS ? cd->aperture : LGPU_APERTURE_NONE;
    cam.blades = cd->blades;
    cam.focal = cd->focal_length;
    cam.ap_size = cd->aperture_size;
    cam.off_phi = cd->offset_phi;
    cam.off_theta = cd->offset_theta;
    if (cam.aperture == LGPU_APERTURE_MASKED) {   /* index checked by check_camera */
        const int t = cd->aperture_mask;
        cam.mask_cond_off = c->mask_cond[t];
        cam.mask_marg_off = c->mask_marg[t];
        cam.mask_w = c->tex_w[t];
        cam.mask_h = c->tex_h[t];
        cam.mask_marg_int = c->mask_int[t];
    }
    return cam;
}

/* Camera parameters a kernel relies on: known type and aperture, a blade count that divides the
 * circle, a masked aperture's texture committed with its distribution, finite lens values. */
int check_camera(lgpu_context *c, const lgpu_camera_desc *cd) {
    if (cd->type < LGPU_CAMERA_PINHOLE || cd->type > LGPU_CAMERA_SPHERICAL) return fail(c, LGPU_ERR_INVALID_ARG, "unknown camera type");
    if (!std::isfinite(cd->fov) || !std::isfinite(cd->offset_phi) || !std::isfinite(cd->offset_theta))
        return fail(c, LGPU_ERR_INVALID_ARG, "camera parameters must be finite");
    if (cd->type != LGPU_CAMERA_THIN_LENS) return LGPU_OK;
    if (!std::isfinite(cd->focal_length) || !std::isfinite(cd->aperture_size)) return fail(c, LGPU_ERR_INVALID_ARG, "lens parameters must be finite");
    if (cd->aperture < LGPU_APERTURE_NONE || cd->aperture > LGPU_APERTURE_MASKED) return fail(c, LGPU_ERR_INVALID_ARG, "unknown aperture type");
    if (cd->aperture == LGPU_APERTURE_BLADE && cd->blades < 1) return fail(c, LGPU_ERR_INVALID_ARG, "a blade aperture needs at least one blade");
    if (cd->aperture == LGPU_APERTURE_MASKED) {
        const int t = cd->aperture_mask;
        if (t < 0 || t >= (int)c->mask_cond.size() || c->mask_cond[t] < 0)
            return fail(c, LGPU_ERR_INVALID_ARG, "masked aperture: texture not committed with aperture_mask set");
    }
    return LGPU_OK;
}

int check_opts(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o) {
    if (!c || !cam || !o) return LGPU_ERR_INVALID_ARG;
    if (!c->have_scene) return fail(c, LGPU_ERR_NO_SCENE, "no committed scene");
    if (o->width <= 0 || o->height <= 0 || o->spp <= 0) return fail(c, LGPU_ERR_INVALID_ARG, "width, height and spp must be positive");
    if (o->max_bounces < 0 || o->min_bounces < 0) return fail(c, LGPU_ERR_INVALID_ARG, "negative bounce count");
    if ((uint64_t)o->width * o->height > (1ull << 32) - 1) return fail(c, LGPU_ERR_INVALID_ARG, "film too large");
    if (o->integrator < LGPU_INTEGRATOR_PATH || o->integrator > LGPU_INTEGRATOR_GPU_MISVOLPATH ||
        o->integrator == LGPU_INTEGRATOR_AOV)
        return fail(c, LGPU_ERR_INVALID_ARG, "integrator not available on the GPU path (AOV passes are not built)");
    return check_camera(c, cam);
}

/* Transmittance walks run inside the trace kernel (WaveArgs::fold_tr) for RGB3 renders, whose
 * spectra the trace kernel computes in; a build with -DLGPU_NO_FOLD_TR keeps one resume per
 * segment for comparison. */
int fold_tr(const lgpu_render_opts *o) {
#ifdef LGPU_NO_FOLD_TR
    (void)o;
    return 0;
#else
    return o->spectral_mode == LGPU_SPECTRAL_RGB3 ? 1 : 0;
#endif
}

/* Kernel launches of one trace step over m queries (the walk segment runs in its own kernel). */
int trace_launches(const WaveArgs &W, int m) {
    const int split = W.fold_tr ? W.seg_off[LG_NSEG - 1] : m;
    return (split > 0 ? 1 : 0) + (m > split ? 1 : 0);
}

/* Grow the wavefront pool to `slots` path slots of `state_bytes` each. */
int ensure_pool(lgpu_context *c, size_t slots, size_t state_bytes, size_t cold_bytes) {
    if (c->w_slots >= slots && c->w_state_bytes == state_bytes) return LGPU_OK;
    cudaFree(c->w_cold);
    c->w_cold = nullptr;
    cudaFree(c->w_states); cudaFree(c->w_qo); cudaFree(c->w_qd); cudaFree(c->w_res); cudaFree(c->w_resobj);
    cudaFree(c->w_qa); cudaFree(c->w_qb); cudaFree(c->w_free); cudaFree(c->w_trout);
    c->w_states = nullptr; c->w_qo = c->w_qd = c->w_res = c->w_trout = nullptr;
    c->w_resobj = c->w_qa = c->w_qb = c->w_free = nullptr;
    c->w_slots = 0;
    cudaError_t e = cudaMalloc(&c->w_states, slots * state_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->w_cold, slots * cold_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->w_qo, slots * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_qd, slots * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_res, slots * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_resobj, slots * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_trout, 2 * slots * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_qa, LG_NSEG * slots * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_qb, LG_NSEG * slots * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->w_free, slots * sizeof(int));
    if (e == cudaSuccess && !c->w_counts) e = cudaMalloc(&c->w_counts, (2 * LG_NSEG + 2) * sizeof(int));
    if (e == cudaSuccess && !c->w_next) e = cudaMalloc(&c->w_next, sizeof(unsigned long long));
    if (e == cudaSuccess && !c->h_count) e = cudaMallocHost(&c->h_count, (2 * LG_NSEG + 2) * sizeof(int));
    for (int k = 0; k < LG_NSEG + 3 && e == cudaSuccess; ++k)
        if (!c->w_ev[k]) e = cudaEventCreate(&c->w_ev[k]);
    if (e != cudaSuccess) return cuda_fail(c, e, "wavefront pool allocation");
    c->w_slots = slots;
    c->w_state_bytes = state_bytes;
    return LGPU_OK;
}

/* Bounce loop as a CUDA graph: two iterations (queue A -> B -> A) of device-driven launches -- the
 * trace, resume and spawn kernels read their queue sizes on the device and run over resident
 * grids -- are captured once per call and replayed; the host reads the queue sizes back only
 * after every second replay to detect the end.  Per-launch timing is not recorded in this mode. */
int run_graph_loop(lgpu_context *c, WaveArgs &W, bool hero, size_t slots, uint64_t n, int tblock, int *qa, int *qb,
                   int *ca, int *cb, cudaStream_t user_st) {
    /* the legacy default stream cannot be captured: work on a stream of the context instead, after
     * everything already queued on the caller's stream (the loop ends synchronised) */
    cudaStream_t st = user_st;
    if (!st) {
        if (!c->graph_stream) {
            cudaError_t e0 = cudaStreamCreateWithFlags(&c->graph_stream, cudaStreamNonBlocking);
            if (e0 != cudaSuccess) return cuda_fail(c, e0, "graph stream");
        }
        cudaError_t e0 = cudaStreamSynchronize(user_st);
        if (e0 != cudaSuccess) return cuda_fail(c, e0, "graph stream");
        st = c->graph_stream;
    }
    auto resume = [&](int m, int mode) { return hero ? wave_resume_4_0(W, m, mode, st) : wave_resume_3_0(W, m, mode, st); };
    cudaError_t e = wave_trace_3_0(W, 0, st, tblock);   /* set-up of the resident grid, before capture */
    if (e != cudaSuccess) return cuda_fail(c, e, "graph set-up");
    const WaveArgs W0 = W;
    auto iteration = [&](int *qin, int *cin, int *qout, int *cout) {
        cudaError_t r = cudaMemsetAsync(cout, 0, LG_NSEG * sizeof(int), st);
        W = W0;
        W.queue_in = qin; W.count_in = cin; W.queue_out = qout; W.count_out = cout; W.cap_in = W.cap;
        if (r == cudaSuccess) r = wave_trace_3_0(W, -1, st, tblock);
        for (int k = 0; k < LG_NSEG && r == cudaSuccess; ++k) { W.seg_sel = k; r = resume(-1, 0); }
        W.seg_sel = 0;
        if (r == cudaSuccess) r = resume(-(int)slots, 1);
        return r;
    };
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t r = iteration(qa, ca, qb, cb);
        if (r == cudaSuccess) r = iteration(qb, cb, qa, ca);
        e = cudaStreamEndCapture(st, &g);
        if (e == cudaSuccess) e = r;
    }
    W = W0;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) { if (ge) cudaGraphExecDestroy(ge); return cuda_fail(c, e, "graph capture"); }
    uint64_t launches = 2, replays = 0;
    int rc = LGPU_OK;
    for (;;) {
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) { e = cudaGraphLaunch(ge, st); ++replays; }
        launches += 2 * 2 * ((W0.fold_tr ? 2 : 1) + LG_NSEG + 2);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_count, ca, LG_NSEG * sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { rc = cuda_fail(c, e, "graph replay"); break; }
        int m = 0;
        for (int k = 0; k < LG_NSEG; ++k) m += c->h_count[k];
        if (m > 0) {
            if (replays > 200000) { rc = fail(c, LGPU_ERR_TIMEOUT, "wavefront did not drain"); break; }
            continue;
        }
        unsigned long long next = 0;
        e = cudaMemcpy(&next, c->w_next, sizeof(next), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { rc = cuda_fail(c, e, "graph replay"); break; }
        if (next >= n) break;
        W.queue_in = nullptr; W.queue_out = qa; W.count_out = ca; W.count_in = nullptr;
        e = resume((int)slots, 2);   /* every slot is idle: spawn into the whole pool again */
        W = W0;
        launches += 2;
        if (e != cudaSuccess) { rc = cuda_fail(c, e, "graph restart"); break; }
    }
    cudaGraphExecDestroy(ge);
    c->stats.iterations += (uint32_t)(2 * replays);
    c->stats.pool_slots = (uint32_t)slots;
    c->stats.spawned += n;
    c->stats.launches += launches;
    return rc ? rc : check_device_error(c, st);
}

/* Run the wavefront over `n` paths (chunk indices 0..n-1 = path ids base.. or ids[]), writing
 * radiance per path into paths_out.  Per iteration: one count read-back, then trace, resume,
 * spawn (new paths into freed slots) and advance. */
int run_wavefront(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o, const uint64_t *ids,
                  uint64_t base, uint64_t n, float4 *paths_out, bool count, cudaStream_t st,
                  const DView *views_dev = nullptr, int n_views = 0) {
    const bool hero = o->spectral_mode == LGPU_SPECTRAL_HERO4;
    const size_t sb = hero ? wave_state_bytes_4_0() : wave_state_bytes_3_0();
    const size_t cbytes = hero ? wave_cold_bytes_4_0() : wave_cold_bytes_3_0();
    /* default pool: 8 Mi slots (~7 GB); on the 1080p terrain 357.4 Mpath-samples/s against 348.3 with
     * 4 Mi (49 bounce iterations instead of 88) */
    const size_t want = o->pool_slots > 0 ? (size_t)o->pool_slots : ((size_t)8 << 20);
    const size_t slots = (size_t)std::min<uint64_t>(n, want);
    if (slots == 0) return LGPU_OK;
    int rc = ensure_pool(c, slots, sb, cbytes);
    if (rc) return rc;
    WaveArgs W;
    std::memset(&W, 0, sizeof(W));
    W.S = c->S;
    W.cam = make_cam(c, cam, o);
    W.rp.spp = o->spp; W.rp.max_bounces = o->max_bounces; W.rp.min_bounces = o->min_bounces;
    W.rp.seed = o->seed; W.rp.sample_offset = o->sample_offset;
    W.states = c->w_states;
    W.cold = c->w_cold;
    W.qo = c->w_qo; W.qd = c->w_qd; W.res = c->w_res; W.res_obj = c->w_resobj;
    W.tr_out = c->w_trout;
    W.fold_tr = fold_tr(o);
    W.next_path = c->w_next;
    W.n_paths = n;
    W.base = base;
    W.ids = ids;
    W.path_out = paths_out;
    W.views = views_dev;
    W.n_views = n_views;
    W.counters = c->d_counters;
    W.cap = (int)slots;
    W.cap_in = (int)slots;
    W.free_list = c->w_free;
    auto resume = [&](int m, int mode) {
        if (hero) return count ? wave_resume_4_1(W, m, mode, st) : wave_resume_4_0(W, m, mode, st);
        return count ? wave_resume_3_1(W, m, mode, st) : wave_resume_3_0(W, m, mode, st);
    };
    int *qa = c->w_qa, *qb = c->w_qb;
    int *ca = c->w_counts, *cb = c->w_counts + LG_NSEG;
    W.free_count = c->w_counts + 2 * LG_NSEG;
    const unsigned long long zero = 0;
    cudaMemcpyAsync(c->w_next, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(c->w_counts, 0, (2 * LG_NSEG + 2) * sizeof(int), st);
    /* first spawn fills the whole pool */
    W.queue_in = nullptr; W.queue_out = qa; W.count_out = ca;
    cudaError_t e = resume((int)slots, 2);
    if (e != cudaSuccess) return cuda_fail(c, e, "wavefront start");
    const int tblock = o->block_size > 0 ? o->block_size : 64;   /* 64 measured fastest on the 1080p terrain */
    if (o->kernel_mode == LGPU_KERNEL_WAVEFRONT_GRAPH && !count)
        return run_graph_loop(c, W, hero, slots, n, tblock, qa, qb, ca, cb, st);
    int iters = 0;
    uint64_t launches = 2;
    /* events around every launch of an iteration: [0] before trace, [1] after trace, [2 + k] after
     * the resume of stage k, [2 + LG_NSEG] after the spawn.  They are read after the next count
     * read-back has synchronised the stream, so timing costs no extra synchronisation. */
    cudaEvent_t *ev = c->w_ev;
    int last_seg[LG_NSEG];
    bool pending = false;
    auto account = [&]() {
        if (!pending) return;
        float t = 0;
        cudaEventElapsedTime(&t, ev[0], ev[1]);
        c->stats.trace_ms += t;
        int prev = 1;
        for (int k = 0; k < LG_NSEG; ++k) {
            if (!last_seg[k]) continue;
            cudaEventElapsedTime(&t, ev[prev], ev[2 + k]);
            c->stats.stage_ms[k] += t;
            c->stats.shade_ms += t;
            prev = 2 + k;
        }
        cudaEventElapsedTime(&t, ev[prev], ev[2 + LG_NSEG]);
        c->stats.spawn_ms += t;
        pending = false;
    };
    for (;;) {
        cudaMemcpyAsync(c->h_count, ca, LG_NSEG * sizeof(int), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(c, e, "wavefront");
        account();
        int m = 0;
        W.seg_off[0] = 0;
        for (int k = 0; k < LG_NSEG; ++k) { m += c->h_count[k]; W.seg_off[k + 1] = m; }
        if (m <= 0) {
            /* no path in flight: done, unless paths that all ended inside a spawn left some unstarted */
            unsigned long long next = 0;
            e = cudaMemcpy(&next, c->w_next, sizeof(next), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cuda_fail(c, e, "wavefront");
            if (next >= n) break;
            W.queue_in = nullptr; W.queue_out = qa; W.count_out = ca;
            e = resume((int)slots, 2);   /* every slot is idle: spawn into the whole pool again */
            if (e != cudaSuccess) return cuda_fail(c, e, "wavefront restart");
            launches += 2;
            continue;
        }
        if (++iters > 100000) return fail(c, LGPU_ERR_TIMEOUT, "wavefront did not drain");
        cudaMemsetAsync(cb, 0, LG_NSEG * sizeof(int), st);
        W.queue_in = qa; W.queue_out = qb; W.count_out = cb;
        cudaEventRecord(ev[0], st);
        e = count ? wave_trace_3_1(W, m, st, tblock) : wave_trace_3_0(W, m, st, tblock);
        cudaEventRecord(ev[1], st);
        c->stats.traced += (uint64_t)m;
        launches += trace_launches(W, m);
        /* one resume launch per queue segment: each launch enters the state machine at one
         * program point, so its warps run the same code */
        const WaveArgs W0 = W;
        for (int k = 0; k < LG_NSEG; ++k) {
            const int nk = W0.seg_off[k + 1] - W0.seg_off[k];
            last_seg[k] = 0;
            if (nk <= 0 || e != cudaSuccess) continue;
            for (int j = 0; j <= LG_NSEG; ++j) W.seg_off[j] = j <= k ? 0 : 0x7fffffff;
            W.queue_in = qa + (size_t)k * W0.cap;
            W.cap_in = 0;
            e = resume(nk, 0);
            cudaEventRecord(ev[2 + k], st);
            last_seg[k] = 1;
            c->stats.resumed[k] += (uint64_t)nk;
            launches += 1;
            W = W0;
        }
        if (e == cudaSuccess) e = resume(m, 1);   /* spawn into the slots freed by this resume */
        cudaEventRecord(ev[2 + LG_NSEG], st);
        launches += 2;
        pending = true;
        if (e != cudaSuccess) return cuda_fail(c, e, "wavefront iteration");
        std::swap(qa, qb);
        std::swap(ca, cb);
    }
    c->last_iterations = iters;
    c->stats.iterations += (uint32_t)iters;
    c->stats.pool_slots = (uint32_t)slots;
    c->stats.spawned += n;
    c->stats.launches += launches;
#ifdef LGPU_STATE_CLOCKS
    {   /* diagnostic build: cycles per program point of this render, to stderr */
        static const char *names[] = {"NEW", "LOOP", "TOP_HIT", "MISS", "BODY", "SURF_A", "SURF_LI", "SURF_EXT",
                                      "NULL_EXT", "RR", "NEXT_ITER", "MED_A", "LDM_START", "LDM_VIS", "LDM_SCAT",
                                      "MED_EXT", "VIS_OCCL", "VIS_TR", "TR_STEP", "DONE"};
        unsigned long long h[32];
        if (cudaMemcpyAsync(h, c->d_counters + 4, sizeof(h), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
            cudaStreamSynchronize(st) == cudaSuccess) {
            std::fprintf(stderr, "state-clock (lane-0 cycles, G):");
            for (int k = 0; k < 20; ++k)
                if (h[k]) std::fprintf(stderr, " %s=%.2f", names[k], (double)h[k] * 1e-9);
            std::fprintf(stderr, "\n");
        }
        cudaMemsetAsync(c->d_counters + 4, 0, 32 * sizeof(unsigned long long), st);
    }
#endif
    return check_device_error(c, st);
}

/* The wavefront state machine is the MIS volumetric integrator; the other integrators run as the
 * megakernel. */
bool use_wavefront(const lgpu_render_opts *o) {
    return o->kernel_mode != LGPU_KERNEL_MEGAKERNEL && o->integrator == LGPU_INTEGRATOR_GPU_MISVOLPATH;
}

int ensure_paths(lgpu_context *c, size_t n) {
    if (c->w_paths_cap >= n) return LGPU_OK;
    cudaFree(c->w_paths);
    c->w_paths = nullptr;
    c->w_paths_cap = 0;
    cudaError_t e = cudaMalloc(&c->w_paths, n * sizeof(float4));
    if (e != cudaSuccess) return cuda_fail(c, e, "per-path buffer");
    c->w_paths_cap = n;
    return LGPU_OK;
}

/* Whole-frame wavefront render into a device film (chunks of whole pixels). */
int wavefront_frame(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o, float4 *film,
                    float4 *paths_all, bool count, cudaStream_t st) {
    const uint64_t px = (uint64_t)o->width * o->height;
    const uint64_t spp = (uint64_t)o->spp;
    const uint64_t max_chunk = (uint64_t)1 << 28;   /* 256 Mi paths = 4 GiB of per-path radiance */
    uint64_t chunk_px = std::max<uint64_t>(1, std::min<uint64_t>(px, max_chunk / spp));
    for (uint64_t p0 = 0; p0 < px; p0 += chunk_px) {
        const uint64_t npx = std::min(chunk_px, px - p0);
        const uint64_t n = npx * spp;
        float4 *out;
        if (paths_all) out = paths_all + p0 * spp;
        else {
            int rc = ensure_paths(c, n);
            if (rc) return rc;
            out = c->w_paths;
        }
        int rc = run_wavefront(c, cam, o, nullptr, p0 * spp, n, out, count, st);
        if (rc) return rc;
        if (film) {
            cudaError_t e = film_reduce(out, film, p0, npx, o->spp, st);
            c->stats.launches += 1;
            if (e != cudaSuccess) return cuda_fail(c, e, "film reduce");
        }
    }
    return LGPU_OK;
}

/* kernel_mode AUTO after lgpu_autotune: the tuned scheme, pool and block size (explicit values in
 * opts win). */
lgpu_render_opts effective_opts(const lgpu_context *c, const lgpu_render_opts *o) {
    lgpu_render_opts r = *o;
    if (r.kernel_mode == LGPU_KERNEL_AUTO && c->tuned) {
        r.kernel_mode = c->tuning.kernel_mode;
        if (r.pool_slots <= 0) r.pool_slots = c->tuning.pool_slots;
        if (r.block_size <= 0) r.block_size = c->tuning.block_size;
    }
    return r;
}

int render_impl(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o_in, float4 *film, float4 *paths,
                const uint64_t *ids, uint64_t n, bool count, cudaStream_t s) {
    const lgpu_render_opts eff = effective_opts(c, o_in);
    const lgpu_render_opts *o = &eff;
    c->stats.trace_ms = c->stats.shade_ms = c->stats.spawn_ms = 0;
    c->stats.iterations = 0;
    for (int k = 0; k < 6; ++k) { c->stats.stage_ms[k] = 0; c->stats.resumed[k] = 0; }
    c->stats.traced = c->stats.spawned = c->stats.launches = 0;
    if (use_wavefront(o)) {
        if (count) cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
        cudaEventRecord(c->ev0, s);
        int rc;
        if (ids) rc = run_wavefront(c, cam, o, ids, 0, n, paths, count, s);
        else rc = wavefront_frame(c, cam, o, film, paths, count, s);
        if (rc) return rc;
        cudaEventRecord(c->ev1, s);
        c->stats.paths = n;
        return LGPU_OK;
    }
    LaunchArgs a;
    a.S = c->S;
    a.cam = make_cam(c, cam, o);
    a.rp.spp = o->spp;
    a.rp.max_bounces = o->max_bounces;
    a.rp.min_bounces = o->min_bounces;
    a.rp.seed = o->seed;
    a.rp.sample_offset = o->sample_offset;
    a.rp.integrator = o->integrator;
    a.film = film;
    a.paths_out = paths;
    a.ids = ids;
    a.n = n;
    a.counters = c->d_counters;
    a.hero = o->spectral_mode == LGPU_SPECTRAL_HERO4;
    a.count = count;
    a.stream = s;
    if (count) cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
    cudaEventRecord(c->ev0, s);
    cudaError_t e = launch_render(a);
    if (e != cudaSuccess) return cuda_fail(c, e, "render launch");
    c->stats.launches += 1;
    cudaEventRecord(c->ev1, s);
    c->stats.paths = n;
    return LGPU_OK;
}

int finish_timing(lgpu_context *c) {
    cudaError_t e = cudaEventSynchronize(c->ev1);
    if (e != cudaSuccess) return cuda_fail(c, e, "render");
    const int rc = check_device_error(c, 0);
    if (rc) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->stats.last_render_ms = ms;
    return LGPU_OK;
}

}  // namespace

extern "C" {

LGPU_API int lgpu_render_device(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o,
                                float *film_dev, float *path_out_dev, void *stream) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    cudaSetDevice(c->device);
    const uint64_t n = (uint64_t)o->width * o->height * o->spp;
    return render_impl(c, cam, o, reinterpret_cast<float4 *>(film_dev), reinterpret_cast<float4 *>(path_out_dev), nullptr, n,
                       false, (cudaStream_t)stream);
}

LGPU_API int lgpu_render(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o, float *film_rgbn) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    if (!film_rgbn) return fail(c, LGPU_ERR_INVALID_ARG, "null film");
    cudaSetDevice(c->device);
    const size_t px = (size_t)o->width * o->height;
    if (c->film_px < px) {
        cudaFree(c->d_film);
        c->d_film = nullptr;
        cudaError_t e = cudaMalloc(&c->d_film, px * sizeof(float4));
        if (e != cudaSuccess) { c->film_px = 0; return cuda_fail(c, e, "film allocation"); }
        c->film_px = px;
    }
    cudaError_t e = cudaMemcpy(c->d_film, film_rgbn, px * sizeof(float4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "film upload");
    const uint64_t n = (uint64_t)px * o->spp;
    r = render_impl(c, cam, o, c->d_film, nullptr, nullptr, n, false, 0);
    if (r) return r;
    r = finish_timing(c);
    if (r) return r;
    e = cudaMemcpy(film_rgbn, c->d_film, px * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "film download");
    return LGPU_OK;
}

LGPU_API int lgpu_render_paths(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o,
                               const uint64_t *path_ids, uint64_t n, float *path_out_host) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    if (!path_ids || !path_out_host) return fail(c, LGPU_ERR_INVALID_ARG, "null path buffers");
    cudaSetDevice(c->device);
    const uint64_t total = (uint64_t)o->width * o->height * o->spp;
    for (uint64_t i = 0; i < n; ++i)
        if (path_ids[i] >= total) return fail(c, LGPU_ERR_INVALID_ARG, "path id out of range");
    if (c->ids_cap < n) {
        cudaFree(c->d_ids);
        c->d_ids = nullptr;
        cudaError_t e = cudaMalloc(&c->d_ids, n * sizeof(uint64_t));
        if (e != cudaSuccess) { c->ids_cap = 0; return cuda_fail(c, e, "id buffer"); }
        c->ids_cap = n;
    }
    if (c->paths_cap < n) {
        cudaFree(c->d_paths);
        c->d_paths = nullptr;
        cudaError_t e = cudaMalloc(&c->d_paths, n * sizeof(float4));
        if (e != cudaSuccess) { c->paths_cap = 0; return cuda_fail(c, e, "path buffer"); }
        c->paths_cap = n;
    }
    cudaError_t e = cudaMemcpy(c->d_ids, path_ids, n * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "id upload");
    r = render_impl(c, cam, o, nullptr, c->d_paths, c->d_ids, n, false, 0);
    if (r) return r;
    r = finish_timing(c);
    if (r) return r;
    e = cudaMemcpy(path_out_host, c->d_paths, n * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "path download");
    return LGPU_OK;
}

LGPU_API int lgpu_render_count(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    cudaSetDevice(c->device);
    const uint64_t n = (uint64_t)o->width * o->height * o->spp;
    r = render_impl(c, cam, o, nullptr, nullptr, nullptr, n, true, 0);
    if (r) return r;
    r = finish_timing(c);
    if (r) return r;
    unsigned long long h[4];
    cudaError_t e = cudaMemcpy(h, c->d_counters, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "counter download");
    c->stats.nodes_visited = h[0];
    c->stats.tris_tested = h[1];
    c->stats.rays = h[2];
    return LGPU_OK;
}

LGPU_API int lgpu_intersect(lgpu_context *c, const float *rays_dev, uint32_t *hits_dev, float *uv_out_dev, uint64_t n, void *stream) {
    if (!c || !rays_dev || !hits_dev) return LGPU_ERR_INVALID_ARG;
    if (!c->have_scene) return fail(c, LGPU_ERR_NO_SCENE, "no committed scene");
    cudaSetDevice(c->device);
    cudaError_t e = launch_intersect(c->S, rays_dev, hits_dev, uv_out_dev, n, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "intersect launch");
    e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "intersect");
    return LGPU_OK;
}

}  // extern "C"

/* ------------------------------------------------------------------ progressive passes, film output */
extern "C" {

LGPU_API int lgpu_film_resolve(const float *film_dev, float *rgba_dev, uint64_t n_px, void *stream) {
    if (!film_dev || !rgba_dev) return LGPU_ERR_INVALID_ARG;
    cudaError_t e = film_resolve(reinterpret_cast<const float4 *>(film_dev), reinterpret_cast<float4 *>(rgba_dev), n_px,
                                 (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    return e == cudaSuccess ? LGPU_OK : LGPU_ERR_CUDA;
}

LGPU_API int lgpu_render_progressive(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o,
                                     int32_t passes, float *film_dev, float *rgba_dev, void *stream) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    if (passes < 0 || !film_dev) return fail(c, LGPU_ERR_INVALID_ARG, "bad progressive pass arguments");
    cudaSetDevice(c->device);
    const uint64_t n = (uint64_t)o->width * o->height * o->spp;
    lgpu_render_opts po = *o;
    for (int p = 0; p < passes; ++p) {
        po.sample_offset = o->sample_offset + (uint32_t)(p * o->spp);   /* the next o->spp samples of every pixel */
        r = render_impl(c, cam, &po, reinterpret_cast<float4 *>(film_dev), nullptr, nullptr, n, false, (cudaStream_t)stream);
        if (r) return r;
        if (rgba_dev) {   /* ProgressiveRender::UpdateOutputTexture after each pass */
            cudaError_t e = film_resolve(reinterpret_cast<const float4 *>(film_dev), reinterpret_cast<float4 *>(rgba_dev),
                                         (uint64_t)o->width * o->height, (cudaStream_t)stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "film resolve");
        }
    }
    return finish_timing(c);
}

}  // extern "C"

/* ------------------------------------------------------------------ batched views
 *
 * lgpu_render_batch renders many views of the committed scene -- each with its own camera, film
 * size, spp, depth and seed -- through one wavefront: consecutive views are packed into chunks of
 * at most 256 Mi paths, a chunk's paths share one pool of path slots, so small views no longer
 * leave the GPU idle and the bounce loop runs once per chunk instead of once per view. */
namespace {

int check_view(lgpu_context *c, const lgpu_view_desc &v) {
    if (v.width <= 0 || v.height <= 0 || v.spp <= 0) return fail(c, LGPU_ERR_INVALID_ARG, "view width, height and spp must be positive");
    if (v.max_bounces < 0) return fail(c, LGPU_ERR_INVALID_ARG, "negative bounce count in a view");
    if ((uint64_t)v.width * v.height > (1ull << 32) - 1) return fail(c, LGPU_ERR_INVALID_ARG, "view film too large");
    if (!v.film_dev) return fail(c, LGPU_ERR_INVALID_ARG, "null view film");
    return check_camera(c, &v.camera);
}

lgpu_render_opts view_opts(const lgpu_render_opts *o, const lgpu_view_desc &v) {
    lgpu_render_opts r = *o;
    r.width = v.width; r.height = v.height; r.spp = v.spp; r.max_bounces = v.max_bounces;
    r.seed = v.seed; r.sample_offset = v.sample_offset;
    return r;
}

/* One chunk of whole views [v0, v1) through one wavefront, then one film reduction per view. */
int batch_chunk(lgpu_context *c, const lgpu_view_desc *views, int v0, int v1, const lgpu_render_opts *o, cudaStream_t st) {
    std::vector<DView> table((size_t)(v1 - v0));
    uint64_t total = 0;
    for (int v = v0; v < v1; ++v) {
        const lgpu_render_opts vo = view_opts(o, views[v]);
        DView &d = table[(size_t)(v - v0)];
        d.cam = make_cam(c, &views[v].camera, &vo);
        d.rp.spp = vo.spp; d.rp.max_bounces = vo.max_bounces; d.rp.min_bounces = vo.min_bounces;
        d.rp.seed = vo.seed; d.rp.sample_offset = vo.sample_offset;
        d.first = total;
        total += (uint64_t)vo.width * vo.height * vo.spp;
    }
    if (c->views_cap < table.size()) {
        cudaFree(c->d_views);
    if (c->graph_stream) cudaStreamDestroy(c->graph_stream);
        c->d_views = nullptr;
        c->views_cap = 0;
        cudaError_t e = cudaMalloc(&c->d_views, table.size() * sizeof(DView));
        if (e != cudaSuccess) return cuda_fail(c, e, "view table");
        c->views_cap = table.size();
    }
    cudaError_t e = cudaMemcpyAsync(c->d_views, table.data(), table.size() * sizeof(DView), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "view table upload");
    int rc = ensure_paths(c, total);
    if (rc) return rc;
    const lgpu_render_opts vo0 = view_opts(o, views[v0]);
    rc = run_wavefront(c, &views[v0].camera, &vo0, nullptr, 0, total, c->w_paths, false, st, c->d_views, v1 - v0);
    if (rc) return rc;
    for (int v = v0; v < v1; ++v) {
        const uint64_t px = (uint64_t)views[v].width * views[v].height;
        e = film_reduce(c->w_paths + table[(size_t)(v - v0)].first, reinterpret_cast<float4 *>(views[v].film_dev), 0, px,
                        views[v].spp, st);
        if (e != cudaSuccess) return cuda_fail(c, e, "film reduce");
        c->stats.launches += 1;
    }
    return LGPU_OK;
}

}  // namespace

extern "C" {

LGPU_API int lgpu_render_batch(lgpu_context *c, const lgpu_view_desc *views, int32_t n_views, const lgpu_render_opts *o_in,
                               void *stream) {
    if (!c || !o_in || n_views < 0 || (n_views > 0 && !views)) return LGPU_ERR_INVALID_ARG;
    const lgpu_render_opts eff = effective_opts(c, o_in);
    const lgpu_render_opts *o = &eff;
    if (!c->have_scene) return fail(c, LGPU_ERR_NO_SCENE, "no committed scene");
    if (o->integrator < LGPU_INTEGRATOR_PATH || o->integrator > LGPU_INTEGRATOR_GPU_MISVOLPATH ||
        o->integrator == LGPU_INTEGRATOR_AOV)
        return fail(c, LGPU_ERR_INVALID_ARG, "integrator not available on the GPU path (AOV passes are not built)");
    if (o->min_bounces < 0) return fail(c, LGPU_ERR_INVALID_ARG, "negative bounce count");
    for (int v = 0; v < n_views; ++v) {
        int r = check_view(c, views[v]);
        if (r) return r;
    }
    cudaSetDevice(c->device);
    cudaStream_t st = (cudaStream_t)stream;
    c->stats.trace_ms = c->stats.shade_ms = c->stats.spawn_ms = 0;
    c->stats.iterations = 0;
    for (int k = 0; k < 6; ++k) { c->stats.stage_ms[k] = 0; c->stats.resumed[k] = 0; }
    c->stats.traced = c->stats.spawned = c->stats.launches = 0;
    cudaEventRecord(c->ev0, st);
    uint64_t all = 0;
    if (o->kernel_mode == LGPU_KERNEL_MEGAKERNEL || o->integrator != LGPU_INTEGRATOR_GPU_MISVOLPATH) {
        /* one megakernel launch per view (the unbatched scheme; the only one for the non-MIS integrators) */
        for (int v = 0; v < n_views; ++v) {
            const lgpu_render_opts vo = view_opts(o, views[v]);
            const uint64_t n = (uint64_t)vo.width * vo.height * vo.spp;
            LaunchArgs a;
            a.S = c->S;
            a.cam = make_cam(c, &views[v].camera, &vo);
            a.rp.spp = vo.spp; a.rp.max_bounces = vo.max_bounces; a.rp.min_bounces = vo.min_bounces;
            a.rp.seed = vo.seed; a.rp.sample_offset = vo.sample_offset; a.rp.integrator = vo.integrator;
            a.film = reinterpret_cast<float4 *>(views[v].film_dev);
            a.paths_out = nullptr; a.ids = nullptr; a.n = n; a.counters = c->d_counters;
            a.hero = vo.spectral_mode == LGPU_SPECTRAL_HERO4;
            a.count = false;
            a.stream = st;
            cudaError_t e = launch_render(a);
            if (e != cudaSuccess) return cuda_fail(c, e, "render launch");
            c->stats.launches += 1;
            all += n;
        }
    } else {
        const uint64_t max_chunk = (uint64_t)1 << 28;
        int v0 = 0;
        uint64_t acc = 0;
        for (int v = 0; v <= n_views; ++v) {
            const uint64_t n = v < n_views ? (uint64_t)views[v].width * views[v].height * views[v].spp : 0;
            if (v == n_views || (acc > 0 && acc + n > max_chunk) || n > max_chunk) {
                if (v > v0 && acc > 0) {
                    int r = batch_chunk(c, views, v0, v, o, st);
                    if (r) return r;
                }
                v0 = v;
                acc = 0;
                if (v < n_views && n > max_chunk) {   /* a view larger than a chunk: pixel chunks of its own */
                    const lgpu_render_opts vo = view_opts(o, views[v]);
                    int r = wavefront_frame(c, &views[v].camera, &vo, reinterpret_cast<float4 *>(views[v].film_dev), nullptr,
                                            false, st);
                    if (r) return r;
                    v0 = v + 1;
                    all += n;
                    continue;
                }
            }
            acc += n;
            all += n;
        }
    }
    cudaEventRecord(c->ev1, st);
    c->stats.paths = all;
    return finish_timing(c);
}

}  // extern "C"

/* ------------------------------------------------------------------ autotuner
 *
 * lgpu_autotune times candidate execution schemes on a probe of the caller's workload (the same
 * views at a reduced spp, into scratch films) and keeps the fastest in the context, where
 * kernel_mode AUTO picks it up: megakernel, host-driven wavefront or graph-replayed wavefront,
 * path-slot pool 2^18 .. 2^22, trace block 64 .. 512 threads. */
extern "C" {

LGPU_API int lgpu_autotune(lgpu_context *c, const lgpu_view_desc *views, int32_t n_views, const lgpu_render_opts *o,
                           int32_t probe_spp, lgpu_tuning *out) {
    if (!c || !o || !views || n_views <= 0 || !out) return LGPU_ERR_INVALID_ARG;
    if (!c->have_scene) return fail(c, LGPU_ERR_NO_SCENE, "no committed scene");
    cudaSetDevice(c->device);
    const int ps = probe_spp > 0 ? probe_spp : 1;
    std::vector<lgpu_view_desc> probe(views, views + n_views);
    uint64_t px = 0, paths = 0;
    for (auto &v : probe) {
        if (v.width <= 0 || v.height <= 0 || v.spp <= 0) return fail(c, LGPU_ERR_INVALID_ARG, "view width, height and spp must be positive");
        v.spp = std::min(v.spp, ps);
        px += (uint64_t)v.width * v.height;
        paths += (uint64_t)v.width * v.height * v.spp;
    }
    float4 *scratch = nullptr;
    cudaError_t e = cudaMalloc(&scratch, px * sizeof(float4));
    if (e != cudaSuccess) return cuda_fail(c, e, "autotune films");
    uint64_t off = 0;
    for (auto &v : probe) { v.film_dev = reinterpret_cast<float *>(scratch + off); off += (uint64_t)v.width * v.height; }
    struct Cand { int mode, pool, block; };
    std::vector<Cand> cands = {{LGPU_KERNEL_MEGAKERNEL, 0, 128}};
    for (int mode : {LGPU_KERNEL_WAVEFRONT, LGPU_KERNEL_WAVEFRONT_GRAPH})
        for (int pool : {1 << 18, 1 << 20, 1 << 22}) {
            if ((uint64_t)pool > 2 * paths && pool != (1 << 18)) continue;   /* larger than the work: same as smaller */
            for (int block : {64, 128, 256, 512}) cands.push_back({mode, pool, block});
        }
    const bool was_tuned = c->tuned;
    c->tuned = false;
    double best = 0;
    Cand bc = cands[0];
    int tried = 0, rc = LGPU_OK;
    for (const Cand &k : cands) {
        lgpu_render_opts t = *o;
        t.kernel_mode = k.mode; t.pool_slots = k.pool; t.block_size = k.block;
        double ms = 0;
        for (int rep = 0; rep < 2 && rc == LGPU_OK; ++rep) {   /* warm-up, then the timed run */
            rc = lgpu_render_batch(c, probe.data(), (int32_t)probe.size(), &t, nullptr);
            ms = c->stats.last_render_ms;
        }
        if (rc) break;
        ++tried;
        const double mps = (double)paths / (ms * 1e-3) / 1e6;
        if (mps > best) { best = mps; bc = k; }
    }
    cudaFree(scratch);
    if (rc) { c->tuned = was_tuned; return rc; }
    c->tuning.kernel_mode = bc.mode;
    c->tuning.pool_slots = bc.pool;
    c->tuning.block_size = bc.block;
    c->tuning.pad = 0;
    c->tuning.mpaths_per_s = best;
    c->tuning.tried = tried;
    c->tuned = true;
    *out = c->tuning;
    return LGPU_OK;
}

}  // extern "C"

/* ------------------------------------------------------------------ path-replay adjoint */
extern "C" {

LGPU_API int lgpu_adjoint(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o,
                          const lgpu_adjoint_desc *p, const float *dloss_dev, float *grad_texture_dev,
                          float *grad_scalars_dev, void *stream) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    if (!p || !dloss_dev || !grad_scalars_dev) return fail(c, LGPU_ERR_INVALID_ARG, "null adjoint buffers");
    if (o->spectral_mode != LGPU_SPECTRAL_RGB3) return fail(c, LGPU_ERR_INVALID_ARG, "the adjoint is implemented for RGB3 only");
    AdjArgs A;
    std::memset(&A, 0, sizeof(A));
    A.dloss = reinterpret_cast<const float4 *>(dloss_dev);
    A.grad_tex = reinterpret_cast<float4 *>(grad_texture_dev);
    A.grad_scalar = grad_scalars_dev;
    A.tex_material = -1; A.rough_material = -1; A.medium = -1;
    if (p->tex_material >= 0) {
        if (p->tex_material >= c->num_materials || p->texture < 0 || p->texture >= (int)c->tex_off.size())
            return fail(c, LGPU_ERR_INVALID_ARG, "adjoint texture or material out of range");
        if (!grad_texture_dev) return fail(c, LGPU_ERR_INVALID_ARG, "null texture gradient");
        A.tex_material = p->tex_material;
        A.tex_off = c->tex_off[p->texture]; A.tex_w = c->tex_w[p->texture]; A.tex_h = c->tex_h[p->texture];
    }
    if (p->rough_material >= c->num_materials) return fail(c, LGPU_ERR_INVALID_ARG, "adjoint roughness material out of range");
    if (p->medium >= c->num_media) return fail(c, LGPU_ERR_INVALID_ARG, "adjoint medium out of range");
    A.rough_material = p->rough_material;
    A.medium = p->medium;
    A.inv_spp = 1.f / (float)o->spp;
    cudaSetDevice(c->device);
    RenderParams rp;
    rp.spp = o->spp; rp.max_bounces = o->max_bounces; rp.min_bounces = o->min_bounces;
    rp.seed = o->seed; rp.sample_offset = o->sample_offset;
    const uint64_t n = (uint64_t)o->width * o->height * o->spp;
    cudaStream_t st = (cudaStream_t)stream;
    cudaEventRecord(c->ev0, st);
    cudaError_t e = launch_adjoint(c->S, make_cam(c, cam, o), rp, A, n, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint launch");
    cudaEventRecord(c->ev1, st);
    c->stats.paths = n;
    c->stats.launches = 1;
    return finish_timing(c);
}

}  // extern "C"

/* ------------------------------------------------------------------ fixed-scratch path render
 *
 * lgpu_render_paths_noalloc runs the same wavefront kernels as lgpu_render_paths, but its whole
 * working set (path-state pool, ray/hit records, stage queues, free list, counters) is carved out
 * of one device array with static storage in this file, and the ids and results live in buffers
 * the caller already owns.  Once the array's address is known the call makes no allocation,
 * device or host: it only issues memsets, kernel launches and small device-to-host reads of the
 * queue counts into a stack array.
 *
 * Layout of the array (each region starts on a 256-byte boundary), for S = LGPU_NOALLOC_MAX_SLOTS:
 *   hot path state   S x max(sizeof PHot<3>, PHot<4>)
 *   cold path state  S x max(sizeof PCold<3>, PCold<4>)
 *   ray origin, ray direction, hit record   3 x S x 16 B
 *   hit object, free list                   2 x S x 4 B
 *   transmittance-walk results              2 x S x 16 B
 *   stage queues A and B                    2 x LG_NSEG x S x 4 B
 *   queue counts, free count                (2 x LG_NSEG + 2) x 4 B
 *   next-path counter                       8 B
 * Only the counts and the next-path counter must be zero when a call starts; the call clears them
 * itself on the caller's stream.  Everything else is written before it is read. */
namespace {

constexpr size_t na_round(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t na_max(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t NA_SLOTS = LGPU_NOALLOC_MAX_SLOTS;
constexpr size_t NA_HOT = na_max(sizeof(PHot<3>), sizeof(PHot<4>));
constexpr size_t NA_COLD = na_max(sizeof(PCold<3>), sizeof(PCold<4>));
constexpr size_t NA_OFF_COLD = na_round(NA_HOT * NA_SLOTS);
constexpr size_t NA_OFF_QO = NA_OFF_COLD + na_round(NA_COLD * NA_SLOTS);
constexpr size_t NA_OFF_QD = NA_OFF_QO + na_round(16 * NA_SLOTS);
constexpr size_t NA_OFF_RES = NA_OFF_QD + na_round(16 * NA_SLOTS);
constexpr size_t NA_OFF_RESOBJ = NA_OFF_RES + na_round(16 * NA_SLOTS);
constexpr size_t NA_OFF_TROUT = NA_OFF_RESOBJ + na_round(4 * NA_SLOTS);
constexpr size_t NA_OFF_FREE = NA_OFF_TROUT + na_round(2 * 16 * NA_SLOTS);
constexpr size_t NA_OFF_QA = NA_OFF_FREE + na_round(4 * NA_SLOTS);
constexpr size_t NA_OFF_QB = NA_OFF_QA + na_round(4 * LG_NSEG * NA_SLOTS);
constexpr size_t NA_OFF_COUNTS = NA_OFF_QB + na_round(4 * LG_NSEG * NA_SLOTS);
constexpr size_t NA_OFF_NEXT = NA_OFF_COUNTS + na_round(4 * (2 * LG_NSEG + 2));
constexpr size_t NA_BYTES = NA_OFF_NEXT + na_round(8);
static_assert(NA_BYTES <= LGPU_NOALLOC_SCRATCH_BYTES, "fixed scratch larger than its stated bound");

__device__ __align__(256) static unsigned char g_na_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex[NA_MAX_DEVICES];
unsigned char *g_na_base[NA_MAX_DEVICES] = {};

}  // namespace

extern "C" {

LGPU_API int lgpu_render_paths_noalloc(lgpu_context *c, const lgpu_camera_desc *cam, const lgpu_render_opts *o,
                                       const uint64_t *path_ids_dev, uint64_t n, float *path_out_dev, void *stream) {
    int r = check_opts(c, cam, o);
    if (r) return r;
    if (n == 0) return LGPU_OK;
    if (!path_ids_dev || !path_out_dev) return fail(c, LGPU_ERR_INVALID_ARG, "null path buffers");
    if (o->kernel_mode == LGPU_KERNEL_MEGAKERNEL)
        return fail(c, LGPU_ERR_INVALID_ARG, "lgpu_render_paths_noalloc runs the wavefront kernels only");
    if (o->integrator != LGPU_INTEGRATOR_GPU_MISVOLPATH)   /* the wavefront is the MIS volumetric integrator */
        return fail(c, LGPU_ERR_INVALID_ARG, "lgpu_render_paths_noalloc runs LGPU_INTEGRATOR_GPU_MISVOLPATH only");
    if (o->pool_slots < 0 || o->pool_slots > LGPU_NOALLOC_MAX_SLOTS) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "pool_slots %d is outside the fixed scratch pool (1..%d slots, 0 = all)",
                      o->pool_slots, LGPU_NOALLOC_MAX_SLOTS);
        return fail(c, LGPU_ERR_INVALID_ARG, msg);
    }
    if (c->device < 0 || c->device >= NA_MAX_DEVICES) return fail(c, LGPU_ERR_INVALID_ARG, "device ordinal out of range");
    const bool hero = o->spectral_mode == LGPU_SPECTRAL_HERO4;
    if ((hero ? wave_state_bytes_4_0() : wave_state_bytes_3_0()) > NA_HOT ||
        (hero ? wave_cold_bytes_4_0() : wave_cold_bytes_3_0()) > NA_COLD)
        return fail(c, LGPU_ERR_INVALID_ARG, "path-state layout larger than the fixed scratch slots");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "set device");
    std::lock_guard<std::mutex> lock(g_na_mutex[c->device]);
    if (!g_na_base[c->device]) {   /* once per device: the address of this device's copy */
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess) return cuda_fail(c, e, "scratch symbol address");
        g_na_base[c->device] = static_cast<unsigned char *>(p);
    }
    unsigned char *base = g_na_base[c->device];
    cudaStream_t st = (cudaStream_t)stream;
    const size_t slots = (size_t)std::min<uint64_t>(n, o->pool_slots > 0 ? (uint64_t)o->pool_slots : NA_SLOTS);

    WaveArgs W;
    std::memset(&W, 0, sizeof(W));
    W.S = c->S;
    W.cam = make_cam(c, cam, o);
    W.rp.spp = o->spp; W.rp.max_bounces = o->max_bounces; W.rp.min_bounces = o->min_bounces;
    W.rp.seed = o->seed; W.rp.sample_offset = o->sample_offset;
    W.states = base;
    W.cold = base + NA_OFF_COLD;
    W.qo = reinterpret_cast<float4 *>(base + NA_OFF_QO);
    W.qd = reinterpret_cast<float4 *>(base + NA_OFF_QD);
    W.res = reinterpret_cast<float4 *>(base + NA_OFF_RES);
    W.res_obj = reinterpret_cast<int *>(base + NA_OFF_RESOBJ);
    W.tr_out = reinterpret_cast<float4 *>(base + NA_OFF_TROUT);
    W.fold_tr = fold_tr(o);
    W.free_list = reinterpret_cast<int *>(base + NA_OFF_FREE);
    W.next_path = reinterpret_cast<unsigned long long *>(base + NA_OFF_NEXT);
    W.n_paths = n;
    W.base = 0;
    W.ids = path_ids_dev;
    W.path_out = reinterpret_cast<float4 *>(path_out_dev);
    W.counters = c->d_counters;
    W.cap = (int)slots;
    W.cap_in = (int)slots;
    int *counts = reinterpret_cast<int *>(base + NA_OFF_COUNTS);
    int *qa = reinterpret_cast<int *>(base + NA_OFF_QA), *qb = reinterpret_cast<int *>(base + NA_OFF_QB);
    int *ca = counts, *cb = counts + LG_NSEG;
    W.free_count = counts + 2 * LG_NSEG;
    auto resume = [&](int m, int mode) { return hero ? wave_resume_4_0(W, m, mode, st) : wave_resume_3_0(W, m, mode, st); };

    /* a failure leaves no work of this call queued against the shared array once the lock is
     * released: drain the stream first (its own error, if any, is already being reported) */
    auto failed = [&](int code, cudaError_t err, const char *what) {
        cudaStreamSynchronize(st);
        return err != cudaSuccess ? cuda_fail(c, err, what) : fail(c, code, what);
    };
    c->stats.trace_ms = c->stats.shade_ms = c->stats.spawn_ms = 0;
    for (int k = 0; k < 6; ++k) { c->stats.stage_ms[k] = 0; c->stats.resumed[k] = 0; }
    c->stats.traced = c->stats.spawned = c->stats.launches = 0;
    c->stats.last_render_ms = 0;
    e = cudaMemsetAsync(counts, 0, (2 * LG_NSEG + 2) * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(W.next_path, 0, sizeof(unsigned long long), st);
    W.queue_in = nullptr; W.queue_out = qa; W.count_out = ca;
    if (e == cudaSuccess) e = resume((int)slots, 2);   /* fill the pool */
    if (e != cudaSuccess) return failed(0, e, "wavefront start");
    int h_count[LG_NSEG];
    int iters = 0;
    /* Every iteration advances each path in flight by at least one query, and one path issues at
     * most (max_bounces + 1) x 2048 + 512 of them (per bounce: an extension query plus up to four
     * transmittance loops of at most 256 segments; at most 256 null-surface crossings per path).
     * So n paths need at most n times that many iterations, whatever the pool size: the bound
     * only catches a state machine that stopped making progress, never a long call. */
    const uint64_t per_path = (uint64_t)(o->max_bounces + 1) * 2048u + 512u;
    const uint64_t max_iters = n > ~0ull / per_path ? ~0ull : n * per_path;
    uint64_t launches = 1;
    for (;;) {
        e = cudaMemcpyAsync(h_count, ca, sizeof(h_count), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return failed(0, e, "wavefront");
        int m = 0;
        W.seg_off[0] = 0;
        for (int k = 0; k < LG_NSEG; ++k) { m += h_count[k]; W.seg_off[k + 1] = m; }
        if (m <= 0) {
            /* no path in flight: done, unless every path of the last spawn ended inside it (e.g.
             * max_bounces = 0) and ids are left unstarted; then spawn into the whole pool again */
            unsigned long long next = 0;
            e = cudaMemcpyAsync(&next, W.next_path, sizeof(next), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return failed(0, e, "wavefront");
            if (next >= n) break;
            if (++iters > max_iters) return failed(LGPU_ERR_TIMEOUT, cudaSuccess, "wavefront did not drain");
            W.queue_in = nullptr; W.queue_out = qa; W.count_out = ca;
            e = resume((int)slots, 2);
            if (e != cudaSuccess) return failed(0, e, "wavefront restart");
            launches += 2;
            continue;
        }
        if (++iters > max_iters) return failed(LGPU_ERR_TIMEOUT, cudaSuccess, "wavefront did not drain");
        e = cudaMemsetAsync(cb, 0, LG_NSEG * sizeof(int), st);
        W.queue_in = qa; W.queue_out = qb; W.count_out = cb;
        if (e == cudaSuccess) e = wave_trace_3_0(W, m, st);
        launches += trace_launches(W, m);
        const WaveArgs W0 = W;
        for (int k = 0; k < LG_NSEG && e == cudaSuccess; ++k) {   /* one resume launch per stage */
            const int nk = W0.seg_off[k + 1] - W0.seg_off[k];
            if (nk <= 0) continue;
            for (int j = 0; j <= LG_NSEG; ++j) W.seg_off[j] = j <= k ? 0 : 0x7fffffff;
            W.queue_in = qa + (size_t)k * W0.cap;
            W.cap_in = 0;
            e = resume(nk, 0);
            c->stats.resumed[k] += (uint64_t)nk;
            launches += 1;
            W = W0;
        }
        if (e == cudaSuccess) e = resume(m, 1);   /* new paths into the freed slots */
        if (e != cudaSuccess) return failed(0, e, "wavefront iteration");
        c->stats.traced += (uint64_t)m;
        launches += 2;
        std::swap(qa, qb);
        std::swap(ca, cb);
    }
    c->stats.paths = n;
    c->stats.spawned = n;
    c->stats.launches = launches;
    c->stats.iterations = (uint32_t)iters;
    c->stats.pool_slots = (uint32_t)slots;
    return check_device_error(c, st);
}

}  // extern "C"
