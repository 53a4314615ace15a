/*
 * Device BVH build (LBVH, after Karras 2012, "Maximizing Parallelism in the Construction of BVHs,
 * Octrees, and k-d Trees"), an alternative to the host's binned-SAH build for the BLAS of a scene:
 *   1. 30-bit Morton codes of the primitive centroids in the centroid bounds;
 *   2. codes sorted on the device (primitive ids as values);
 *   3. the binary radix tree over the sorted codes, one thread per inner node: the node's range
 *      direction from its neighbours' common prefixes, the range end and the split by binary
 *      searches (equal codes are told apart by their indices);
 *   4. boxes reduced bottom-up: every leaf thread climbs, and at each inner node the second child to
 *      arrive (an atomic counter per node) computes the union and goes on;
 *   5. the module's binary node records (DNode: both child boxes in the parent), one primitive per
 *      leaf, in the node/primitive numbering of the host build.
 * Same traversal, same node layout; the tree is shallower in quality than SAH (more node visits per
 * ray) and is built in milliseconds instead of seconds.
 */
#include <cuda_runtime.h>

#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "lgpu_build.h"

namespace lg {
namespace {

/* 10 bits spread to every third bit */
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_morton(const float4 *lo, const float4 *hi, int n, float3 cmin, float3 cscale, uint32_t *keys,
                         uint32_t *vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = lo[i], b = hi[i];
    const float cx = ((a.x + b.x) * .5f - cmin.x) * cscale.x;
    const float cy = ((a.y + b.y) * .5f - cmin.y) * cscale.y;
    const float cz = ((a.z + b.z) * .5f - cmin.z) * cscale.z;
    const uint32_t x = (uint32_t)fminf(fmaxf(cx * 1024.f, 0.f), 1023.f);
    const uint32_t y = (uint32_t)fminf(fmaxf(cy * 1024.f, 0.f), 1023.f);
    const uint32_t z = (uint32_t)fminf(fmaxf(cz * 1024.f, 0.f), 1023.f);
    keys[i] = (spread10(x) << 2) | (spread10(y) << 1) | spread10(z);
    vals[i] = (uint32_t)i;
}

/* common-prefix length of sorted codes i and j; -1 outside [0, n) */
__device__ __forceinline__ int prefix(const uint32_t *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = k[i], b = k[j];
    return a == b ? 32 + __clz((uint32_t)(i ^ j)) : __clz(a ^ b);
}

/* inner node i of n - 1: children as refs (>= 0 inner node, < 0 leaf -(j + 1)), parents of both */
__global__ void k_radix_tree(const uint32_t *k, int n, int2 *child, int *parent_inner, int *parent_leaf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = prefix(k, n, i, i + 1) - prefix(k, n, i, i - 1) > 0 ? 1 : -1;
    const int dmin = prefix(k, n, i, i - d);
    int lmax = 2;
    for (int g = 0; g < 31 && prefix(k, n, i, i + lmax * d) > dmin; ++g) lmax *= 2;   /* ends by 2n: -1 outside */
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (prefix(k, n, i, i + (l + t) * d) > dmin) l += t;
    /* l >= 1: with codes made unique by their positions, the neighbour in direction d shares the
     * longer prefix; the guard below only bounds the loop */
    const int j = i + l * d;
    const int dnode = prefix(k, n, i, j);
    int s = 0;
    for (int t = l, g = 0; g < 32; ++g) {
        t = (t + 1) / 2;
        if (prefix(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = lo == gamma ? -(gamma + 1) : gamma;
    const int right = hi == gamma + 1 ? -(gamma + 2) : gamma + 1;
    child[i] = make_int2(left, right);
    if (left < 0) parent_leaf[gamma] = i; else parent_inner[gamma] = i;
    if (right < 0) parent_leaf[gamma + 1] = i; else parent_inner[gamma + 1] = i;
}

/* leaf j (sorted order) holds primitive vals[j] */
__global__ void k_bounds(const float4 *plo, const float4 *phi, const uint32_t *vals, int n, const int2 *child,
                         const int *parent_inner, const int *parent_leaf, float4 *nlo, float4 *nhi,
                         unsigned int *arrivals) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int p = parent_leaf[j];
    for (int guard = 0; p >= 0 && guard < n; ++guard) {
        __threadfence();   /* this child's box (a node box written below) before the arrival count */
        if (atomicAdd(&arrivals[p], 1u) == 0) return;   /* the sibling finishes this node */
        const int2 c = child[p];
        float4 alo, ahi, blo, bhi;
        if (c.x < 0) { const uint32_t q = vals[-c.x - 1]; alo = plo[q]; ahi = phi[q]; }
        else { alo = __ldcg(&nlo[c.x]); ahi = __ldcg(&nhi[c.x]); }
        if (c.y < 0) { const uint32_t q = vals[-c.y - 1]; blo = plo[q]; bhi = phi[q]; }
        else { blo = __ldcg(&nlo[c.y]); bhi = __ldcg(&nhi[c.y]); }
        __stcg(&nlo[p], make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.f));
        __stcg(&nhi[p], make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.f));
        p = parent_inner[p];
    }
}

/* inner node i -> DNode: child c's box is (xs[2c], xs[2c + 1]) etc., refs (index << 4) | count */
__global__ void k_emit(const float4 *plo, const float4 *phi, const uint32_t *vals, int n, const int2 *child,
                       const float4 *nlo, const float4 *nhi, int node_base, int prim_base, DNode *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int2 c = child[i];
    float4 alo, ahi, blo, bhi;
    int ra, rb;
    if (c.x < 0) { const int j = -c.x - 1; alo = plo[vals[j]]; ahi = phi[vals[j]]; ra = ((prim_base + j) << 4) | 1; }
    else { alo = __ldcg(&nlo[c.x]); ahi = __ldcg(&nhi[c.x]); ra = (node_base + c.x) << 4; }
    if (c.y < 0) { const int j = -c.y - 1; blo = plo[vals[j]]; bhi = phi[vals[j]]; rb = ((prim_base + j) << 4) | 1; }
    else { blo = __ldcg(&nlo[c.y]); bhi = __ldcg(&nhi[c.y]); rb = (node_base + c.y) << 4; }
    DNode d;
    d.xs = make_float4(alo.x, ahi.x, blo.x, bhi.x);
    d.ys = make_float4(alo.y, ahi.y, blo.y, bhi.y);
    d.zs = make_float4(alo.z, ahi.z, blo.z, bhi.z);
    d.ch = make_int4(ra, rb, 0, 0);
    out[i] = d;
}

}  // namespace

int build_lbvh_device(const std::vector<Aabb> &boxes, int node_base, int prim_base, BvhOut &out, float *device_ms,
                      std::string &err) {
    const int n = (int)boxes.size();
    out.nodes.clear();
    out.order.clear();
    out.max_depth = 0;
    if (n < 2) { err = "device build needs at least two primitives"; return 1; }
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    std::vector<float4> lo(n), hi(n);
    for (int i = 0; i < n; ++i) {
        const Aabb &b = boxes[i];
        lo[i] = make_float4(b.lo[0], b.lo[1], b.lo[2], 0.f);
        hi[i] = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.f);
        for (int a = 0; a < 3; ++a) {
            const float c = (b.lo[a] + b.hi[a]) * .5f;
            cmin[a] = std::min(cmin[a], c);
            cmax[a] = std::max(cmax[a], c);
        }
    }
    float scale[3];
    for (int a = 0; a < 3; ++a) scale[a] = cmax[a] > cmin[a] ? 1.f / (cmax[a] - cmin[a]) : 0.f;

    float4 *plo = nullptr, *phi = nullptr, *nlo = nullptr, *nhi = nullptr;
    uint32_t *keys = nullptr, *vals = nullptr;
    int2 *child = nullptr;
    int *pin = nullptr, *pleaf = nullptr;
    unsigned int *arrivals = nullptr;
    DNode *dn = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaSuccess;
    auto A = [&](void **p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes); };
    A((void **)&plo, n * sizeof(float4)); A((void **)&phi, n * sizeof(float4));
    A((void **)&nlo, (n - 1) * sizeof(float4)); A((void **)&nhi, (n - 1) * sizeof(float4));
    A((void **)&keys, n * sizeof(uint32_t)); A((void **)&vals, n * sizeof(uint32_t));
    A((void **)&child, (n - 1) * sizeof(int2)); A((void **)&pin, (n - 1) * sizeof(int)); A((void **)&pleaf, n * sizeof(int));
    A((void **)&arrivals, (n - 1) * sizeof(unsigned int)); A((void **)&dn, (n - 1) * sizeof(DNode));
    if (e == cudaSuccess) e = cudaMemcpy(plo, lo.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(phi, hi.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int bs = 256, gl = (n + bs - 1) / bs, gi = (n - 1 + bs - 1) / bs;
    if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
    if (e == cudaSuccess) {
        k_morton<<<gl, bs>>>(plo, phi, n, make_float3(cmin[0], cmin[1], cmin[2]), make_float3(scale[0], scale[1], scale[2]),
                             keys, vals);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        thrust::sort_by_key(thrust::device, thrust::device_ptr<uint32_t>(keys), thrust::device_ptr<uint32_t>(keys) + n,
                            thrust::device_ptr<uint32_t>(vals));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemset(pin, 0xff, (n - 1) * sizeof(int));   /* -1: the root has no parent */
    if (e == cudaSuccess) e = cudaMemset(arrivals, 0, (n - 1) * sizeof(unsigned int));
    if (e == cudaSuccess) { k_radix_tree<<<gi, bs>>>(keys, n, child, pin, pleaf); e = cudaGetLastError(); }
    if (e == cudaSuccess) {
        k_bounds<<<gl, bs>>>(plo, phi, vals, n, child, pin, pleaf, nlo, nhi, arrivals);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_emit<<<gi, bs>>>(plo, phi, vals, n, child, nlo, nhi, node_base, prim_base, dn);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) {
        out.nodes.resize(n - 1);
        out.order.resize(n);
        e = cudaMemcpy(out.nodes.data(), dn, (n - 1) * sizeof(DNode), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(out.order.data(), vals, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(plo); cudaFree(phi); cudaFree(nlo); cudaFree(nhi); cudaFree(keys); cudaFree(vals);
    cudaFree(child); cudaFree(pin); cudaFree(pleaf); cudaFree(arrivals); cudaFree(dn);
    if (e != cudaSuccess) {
        err = std::string("device BVH build: ") + cudaGetErrorString(e);
        out.nodes.clear();
        out.order.clear();
        return 2;
    }
    /* depth of the tree (levels of inner nodes), for the scene report */
    std::vector<int> depth(n - 1, 0);
    int maxd = 1;
    std::vector<int> stack(1, 0);
    depth[0] = 1;
    while (!stack.empty()) {
        const int k = stack.back();
        stack.pop_back();
        maxd = std::max(maxd, depth[k]);
        const int4 c = out.nodes[k].ch;
        for (int r : {c.x, c.y})
            if ((r & 15) == 0) {
                const int idx = (r >> 4) - node_base;
                if (idx <= 0 || idx >= n - 1) { err = "device BVH build: bad child"; return 3; }
                depth[idx] = depth[k] + 1;
                stack.push_back(idx);
            }
    }
    out.max_depth = maxd;
    out.root_ref = node_base << 4;
    if (device_ms) *device_ms = ms;
    return 0;
}

}  // namespace lg
