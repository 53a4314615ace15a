/*
 * Wavefront form of MISVolumetricPathIntegrator::Li (src/integrators/MISVolumetricPathIntegrator.cpp:23-215).
 *
 * The integrator is cut at every ray query into a resumable state machine.  A pool of path slots
 * lives in HBM (PHot + PCold, one per slot); each iteration of the host loop runs
 *   k_trace   -- every pending query (closest hit or occlusion) with a small, register-light
 *                traversal kernel, queries read from a compacted queue;
 *   k_resume  -- every slot with an answered query continues its path until it issues the next
 *                query (appended to the next queue with warp-aggregated atomics) or finishes; a
 *                finished slot writes its radiance and immediately starts the next path id
 *                (path regeneration), so the pool stays full until the frame runs out of paths.
 * The order of random-number draws and every arithmetic step are those of the megakernel and the
 * CPU oracle, so results match them path for path.  Scene::IntersectTr loops (null surfaces,
 * medium boundaries, transmittance) are a sub-machine that issues one closest-hit query per segment.
 */
#pragma once
#include <cooperative_groups.h>
#include "lgpu_camera.cuh"
#include "lgpu_integrator.cuh"
#include "lgpu_launch.h"

namespace lg {

namespace cgx = cooperative_groups;

/* Query types (low byte of the direction record's w; a transmittance walk keeps its medium + 1 in
 * the bits above). */
enum : int { Q_CLOSEST = 1, Q_OCCL = 2, Q_TR = 3 };

enum : int {
    PC_NEW = 0, PC_LOOP, PC_TOP_HIT, PC_MISS, PC_BODY, PC_SURF_A, PC_SURF_LI, PC_SURF_EXT, PC_NULL_EXT,
    PC_RR, PC_NEXT_ITER, PC_MED_A, PC_LDM_START, PC_LDM_VIS, PC_LDM_SCAT, PC_MED_EXT,
    PC_VIS_OCCL, PC_VIS_TR, PC_TR_STEP, PC_DONE
};
enum : int { VIS_AREA = 0, VIS_POINT = 1, VIS_ESCAPE = 2 };

/* Queue segments: slots waiting on a query are grouped by the program point that resumes them, so a
 * warp of k_resume mostly runs one branch of the state machine and k_trace sees closest-hit and
 * occlusion queries in separate runs. */
#define LG_NSEG 6
__host__ __device__ __forceinline__ int seg_of(int pc) {
    switch (pc) {
    case PC_TOP_HIT: return 0;
    case PC_SURF_EXT: return 1;
    case PC_NULL_EXT: return 2;
    case PC_MED_EXT: return 3;
    case PC_VIS_OCCL: return 4;
    default: return 5;   /* PC_TR_STEP */
    }
}
enum : int { TR_TEMP = 0, TR_EVENT = 1 };

/* Per-slot path state.  The hot part (everything a surface bounce touches) is staged through
 * shared memory by k_resume with coalesced warp copies; the cold part (medium bounce and the
 * IntersectTr sub-machine) stays in HBM and is only touched by paths inside participating media. */
template <int NS>
struct __align__(16) PHot {
    uint64_t out;                 /* output index of the path (within the chunk) */
    uint32_t key, dim;
    uint32_t pixel, view;         /* view: index into WaveArgs::views (batched renders) */
    float lam[4];
    int pc, bounces, nullCrossings, scatterIntersect;
    Spec<NS> L, beta;
    float3 ro, rd;
    RayHit hit;
    Event ev;
    /* surface bounce */
    LRef l;
    float lightDistPdf, scatteringPDF, lightPDF, lsSinT;
    float3 sp, sn;
    Spec<NS> Ld, f;
    float3 lsP;                   /* light point (area/point) or env (u, v) */
    int lsT;                      /* sampled triangle of a mesh light */
    /* visibility sub-machine */
    int visRet, visMode, visOK;
    float visM;
    Spec<NS> trTr;                /* transmittance of the last visibility / IntersectTr query */
    float tmpTFar;
    int trResult;
    int pad1, pad2;
};
template <int NS>
struct __align__(16) PCold {
    /* medium bounce */
    LRef ml;
    float3 mPoint, mNormal;
    Spec<NS> mLe;
    float mPdf;
    int choice, medK;
    float distT, distPdf, eqT, eqPdf, distW, eqW;
    Spec<NS> mTrD, mTrE, mLd, kLd;
    float3 mpD, mpE, wiD, wiE;
    float kPartial, kPhasePdf;
    /* IntersectTr sub-machine */
    int trRet, trTarget, trMed, trIter;
    float trTFar, trMaxT;
    float3 trO, trD;
};

/* bulk copies move whole records: sizes must be multiples of 16 bytes */
static_assert(sizeof(PHot<3>) % 16 == 0 && sizeof(PHot<4>) % 16 == 0, "path-state record not 16-byte sized");

struct WaveArgs {
    DeviceScene S;
    CamParams cam;
    RenderParams rp;
    void *states;                 /* PHot per slot */
    void *cold;                   /* PCold per slot */
    float4 *qo, *qd;              /* per slot: origin + tmax, direction + query type */
    float4 *res;                  /* per slot: t, u, v, prim (closest) or occluded flag */
    int *res_obj;
    const int *queue_in;          /* LG_NSEG segments of `cap` entries */
    int *queue_out;
    int *count_out;               /* LG_NSEG counters of queue_out */
    int seg_off[LG_NSEG + 1];     /* prefix offsets of the queue_in segments */
    int cap;                      /* capacity of one queue_out segment */
    int cap_in;                   /* stride between queue_in segments */
    int *free_list;               /* slots whose path ended this iteration */
    int *free_count;
    unsigned long long *next_path;
    uint64_t n_paths;             /* paths in this chunk */
    uint64_t base;                /* path id of chunk index 0 (when ids == nullptr) */
    const uint64_t *ids;          /* explicit path ids or nullptr */
    float4 *path_out;             /* radiance per chunk index, w = random numbers drawn */
    const DView *views;           /* batched views of this chunk (nullptr: one view, cam + rp) */
    int n_views;
    /* Device-driven launches (bounce loop captured in a CUDA graph): the kernels read the sizes of
     * the input queue segments from count_in instead of taking them from the host (seg_off, n). */
    const int *count_in;
    int seg_sel;                  /* device-driven resume: the one segment this launch continues */
    unsigned long long *counters; /* traversal counters (COUNT variant) */
    /* Transmittance walks folded into the trace kernel (RGB3 renders): a Q_TR query runs the whole
     * Scene::IntersectTr loop there and leaves, per slot, tr_out[2 slot] = (Tr, accumulated
     * distance) and tr_out[2 slot + 1] = (origin of the last segment, flags: 1 = stopped on a
     * surface, 2 = a segment was hit), with the last segment's hit in res / res_obj. */
    float4 *tr_out;
    int fold_tr;
};

#ifdef LGPU_STATE_CLOCKS
/* Diagnostic build: SM cycles spent in each program point of Wave::run, sampled on lane 0 of every
 * warp and added into clk[pc] (the context's counter block past the traversal counters). */
struct StateClock {
    unsigned long long *clk;
    int pc = -1;
    long long t = 0;
    bool on;
    __device__ explicit StateClock(unsigned long long *c) : clk(c), on(c && (threadIdx.x & 31) == 0) {}
    __device__ void tick(int next) {
        if (!on) return;
        const long long now = clock64();
        if (pc >= 0 && pc < 32) atomicAdd(&clk[pc], (unsigned long long)(now - t));
        pc = next;
        t = now;
    }
    __device__ ~StateClock() { tick(-1); }
};
#endif

/* Append `slot` to segment `seg` of the next queue; one atomic per group of lanes with the same
 * segment. */
__device__ __forceinline__ void push_queue(const WaveArgs &W, int slot, int seg) {
    cgx::coalesced_group all = cgx::coalesced_threads();
    cgx::coalesced_group g = cgx::labeled_partition(all, seg);
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(W.count_out + seg, (int)g.size());
    base = g.shfl(base, 0);
    W.queue_out[seg * W.cap + base + g.thread_rank()] = slot;
}
__device__ __forceinline__ void push_free(const WaveArgs &W, int slot) {
    cgx::coalesced_group g = cgx::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(W.free_count, (int)g.size());
    base = g.shfl(base, 0);
    W.free_list[base + g.thread_rank()] = slot;
}

template <int NS, bool COUNT>
struct Wave {
    const WaveArgs &W;
    PHot<NS> &s;
    PCold<NS> &c;
    int slot;
    Rng rng;
    Lambda4 lam;
    TravStats st;

    __device__ Tracer<NS, COUNT> T() { return Tracer<NS, COUNT>{W.S, rng, lam, &st}; }

    __device__ void issue(float3 o, float3 d, float tmax, int type, int next) {
        W.qo[slot] = make_float4(o.x, o.y, o.z, tmax);
        W.qd[slot] = make_float4(d.x, d.y, d.z, __int_as_float(type));
        s.pc = next;
        push_queue(W, slot, seg_of(next));
    }
    /* result of the last closest query: valid hit as Scene::Intersect defines it */
    __device__ bool closest(HitRec &hr) {
        const float4 r = W.res[slot];
        hr.t = r.x; hr.u = r.y; hr.v = r.z; hr.prim = __float_as_int(r.w); hr.obj = W.res_obj[slot];
        return hr.obj >= 0 && hr.t > 0.f && hr.t < finf();
    }
    __device__ bool occluded() { return W.res[slot].x != 0.f; }

    /* ---- sub-machines ---- */
    __device__ void start_tr(float3 o, float3 d, int med, int target, float maxT, int ret) {
        c.trO = o; c.trD = d; c.trMed = med; c.trTarget = target; c.trMaxT = maxT; c.trRet = ret;
        c.trTFar = 0.f; c.trIter = 0; s.trTr = Spec<NS>(1.f);
        if (target == TR_TEMP) s.tmpTFar = finf();
        if (NS == 3 && W.fold_tr) issue(o, d, maxT, Q_TR | ((med + 1) << 8), PC_TR_STEP);   /* the whole walk */
        else issue(o, d, finf(), Q_CLOSEST, PC_TR_STEP);
    }
    /* Light::MutualVisibility / PointMutualVisibility / RayEscapes (Light.cpp:10-49) */
    __device__ void start_vis(float3 o, float3 d, float m, int mode, int ret) {
        s.visRet = ret; s.visMode = mode; s.visM = m; s.trTr = Spec<NS>(1.f);
        if (!W.S.has_volumes) {
            issue(o, d, mode == VIS_ESCAPE ? finf() : (float)(m - .00001), Q_OCCL, PC_VIS_OCCL);
        } else {
            start_tr(o, d, s.ev.medium, TR_TEMP, mode == VIS_POINT ? m : -1.f, PC_VIS_TR);
        }
    }

    /* Light::Sample_Li up to its visibility query (MeshLight.cpp:22-42, :134-151, PointLight.cpp:18-29,
     * Spotlight.cpp:44-55, EnvironmentLight.cpp:24-45).  Returns false when no query is needed (the
     * sample already failed, lightPDF = 0). */
    __device__ bool li_prepare() {
        const DeviceScene &S = W.S;
        s.lightPDF = 0.f;
        if (s.l.light < 0) return false;
        const DLight &L = S.lights[s.l.light];
        auto t = T();
        if (L.type == LT_ENV) {
            const DEnv &E = S.env;
            const float u0 = rng.next(), u1 = rng.next();
            float pm, pc; int row;
            const float d1 = t.p1d_sample_cont(E.marg_off, E.h, E.marg_integral, u1, &pm, &row);
            const int co = E.cond_off + row * (2 * E.w + 2);
            const float d0 = t.p1d_sample_cont(co, E.w, S.fpool[co + 2 * E.w + 1], u0, &pc, nullptr);
            s.lightPDF = pc * pm;
            if (s.lightPDF == 0.f) return false;
            const float theta = d1 * PI + E.offy, phi = d0 * PI2 + E.offx;
            const float cT = cosf(theta), sT = sinf(theta);
            if (sT == 0.f) { s.lightPDF = 0.f; return false; }
            s.ev.wi = spherical_dir(sT, cT, phi);
            s.lsP = mk(d0, d1, 0.f);
            s.lsSinT = sT;
            start_vis(s.hit.point + s.hit.nG * SURFACE_EPSILON, s.ev.wi, 0.f, VIS_ESCAPE, PC_SURF_LI);
            return true;
        }
        if (L.type == LT_POINT || L.type == LT_SPOT) {
            const float3 p = s.hit.point + s.hit.nG * SURFACE_EPSILON * (float)s.ev.sidedness;
            const float3 diff = L.pos - p;
            const float m = mag(diff);
            s.ev.wi = divs(diff, m);
            start_vis(p, s.ev.wi, m, VIS_POINT, PC_SURF_LI);
            return true;
        }
        int tri = s.l.tri;
        float u0, u1;
        if (tri < 0) {
            tri = t.mesh_pick(L, rng.next(), &s.lightPDF);
            u0 = rng.next(); u1 = rng.next();
        } else {
            u0 = rng.next(); u1 = rng.next();
        }
        float3 a, b, c;
        t.tri_verts(L, tri, a, b, c);
        const float3 pL = a + (b - a) * u0 + (c - a) * u1;
        const float3 pS = s.hit.point + s.hit.nG * SURFACE_EPSILON * (float)s.ev.sidedness;
        const float3 diff = pL - pS;
        const float m = mag(diff);
        s.ev.wi = divs(diff, m);
        s.lsP = pL;
        s.lsT = tri;
        start_vis(pS, s.ev.wi, m, VIS_AREA, PC_SURF_LI);
        return true;
    }
    /* the rest of Light::Sample_Li once visibility is known */
    __device__ Spec<NS> li_complete() {
        const DeviceScene &S = W.S;
        const DLight &L = S.lights[s.l.light];
        auto t = T();
        const Spec<NS> Tr = s.trTr;
        if (L.type == LT_ENV) {
            if (s.visOK) {
                s.ev.wiL = ev_local(s.hit, s.ev.wi);
                s.lightPDF /= 2.f * PI * PI * s.lsSinT;
                return t.env_texel_uv(s.lsP.x, s.lsP.y) * Tr * S.env.intensity;
            }
            s.lightPDF = 0.f;
            return Spec<NS>(0.f);
        }
        if (L.type == LT_POINT || L.type == LT_SPOT) {
            if (s.visOK) {
                s.lightPDF = 1.f;
                const float d2 = distsq(L.pos, s.hit.point);
                s.ev.wiL = ev_local(s.hit, s.ev.wi);
                Spec<NS> e = t.emission(L, s.ev, s.hit, false) * Tr;
                if (L.type == LT_SPOT) e = e * t.spot_falloff(L, -s.ev.wi);
                return e * L.intensity / d2;
            }
            s.lightPDF = 0.f;
            return Spec<NS>(0.f);
        }
        if (s.visOK) {
            float3 a, b, c;
            t.tri_verts(L, s.lsT, a, b, c);
            float area; float3 n;
            Tracer<NS, COUNT>::area_normal(a, b, c, &area, &n);
            const float cT = fabsf(dot(n, -s.ev.wi));
            if (cT > 0.f) {
                s.ev.wiL = ev_local(s.hit, s.ev.wi);
                if (s.l.tri < 0) s.lightPDF *= distsq(s.hit.point, s.lsP) / (cT * area);
                else s.lightPDF = distsq(s.hit.point, s.lsP) / (cT * area);   /* B10 */
                return t.emission(L, s.ev, s.hit, true) * Tr * L.intensity * INV_PI;
            }
        }
        s.lightPDF = 0.f;
        return Spec<NS>(0.f);
    }
    /* Light::Visibility for a medium point (LdMediumPoint): query part */
    __device__ void ldm_vis_prepare(float3 p) {
        const DeviceScene &S = W.S;
        if (c.ml.light < 0) { c.mPdf = 0.f; s.visOK = 0; s.pc = PC_LDM_VIS; s.visMode = -1; return; }
        const DLight &L = S.lights[c.ml.light];
        if (L.type == LT_ENV) {
            const float3 wi = normalised(c.mPoint - p);
            start_vis(p, wi, 0.f, VIS_ESCAPE, PC_LDM_VIS);
            return;
        }
        if (L.type == LT_POINT || L.type == LT_SPOT) {
            const float3 q = p + s.hit.nG * SURFACE_EPSILON * (float)s.ev.sidedness;
            const float3 diff = c.mPoint - q;
            const float m = mag(diff);
            s.ev.wi = divs(diff, m);
            start_vis(q, s.ev.wi, m, VIS_POINT, PC_LDM_VIS);
            return;
        }
        const float3 diff = c.mPoint - p;
        const float m = mag(diff);
        s.ev.wi = divs(diff, m);
        start_vis(p, s.ev.wi, m, VIS_AREA, PC_LDM_VIS);
    }
    __device__ Spec<NS> ldm_vis_complete(float3 p) {
        const DeviceScene &S = W.S;
        if (c.ml.light < 0) { c.mPdf = 0.f; return Spec<NS>(0.f); }
        const DLight &L = S.lights[c.ml.light];
        auto t = T();
        const Spec<NS> Tr = s.trTr;
        if (!s.visOK) { c.mPdf = 0.f; return Spec<NS>(0.f); }
        if (L.type == LT_ENV) return Tr;
        if (L.type == LT_POINT || L.type == LT_SPOT) {
            Spec<NS> v = Tr;
            if (L.type == LT_SPOT) v = v * t.spot_falloff(L, -s.ev.wi);
            return v / distsq(L.pos, s.hit.point);
        }
        const float cT = c.ml.tri < 0 ? fabsf(dot(c.mNormal, -s.ev.wi)) : fabsf(dot(s.hit.nG, -s.ev.wi));
        c.mPdf *= distsq(p, c.mPoint) / cT;
        return Tr;
    }

    __device__ void finish() {
        float rgb[3];
        const Spec<NS> L = s.L;
        if (NS == 3) { rgb[0] = L.c[0]; rgb[1] = L.c[1]; rgb[2] = L.c[2]; }
        else {
            float xyz[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float w = L.c[i] * (HERO_RANGE / (4.0f * LGPU_CIE_Y_INTEGRAL));
                xyz[0] += w * cie_at(d_cie_x, lam.l[i]);
                xyz[1] += w * cie_at(d_cie_y, lam.l[i]);
                xyz[2] += w * cie_at(d_cie_z, lam.l[i]);
            }
            rgb[0] = 3.240479f * xyz[0] - 1.537150f * xyz[1] - 0.498535f * xyz[2];
            rgb[1] = -0.969256f * xyz[0] + 1.875991f * xyz[1] + 0.041556f * xyz[2];
            rgb[2] = 0.055648f * xyz[0] - 0.204043f * xyz[1] + 1.057311f * xyz[2];
        }
        W.path_out[s.out] = make_float4(rgb[0], rgb[1], rgb[2], (float)rng.dim);
    }

    /* Start path number `idx` of the chunk in this slot (camera ray, Render.cpp:55-56 + Camera.cpp:41-71). */
    __device__ void start_path(uint64_t idx) {
        int view = 0;
        uint64_t pid;
        if (W.views) {
            /* last view whose first path is <= idx (views are in path order) */
            int lo = 0, hi = W.n_views - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (W.views[mid].first <= idx) lo = mid; else hi = mid - 1;
            }
            view = lo;
            pid = idx - W.views[view].first;
        } else {
            pid = W.ids ? W.ids[idx] : W.base + idx;
        }
        const RenderParams &rp = W.views ? W.views[view].rp : W.rp;
        const CamParams &cam = W.views ? W.views[view].cam : W.cam;
        s.view = (uint32_t)view;
        const uint32_t pixel = (uint32_t)(pid / (uint64_t)rp.spp);
        const uint32_t sidx = (uint32_t)(pid % (uint64_t)rp.spp) + rp.sample_offset;
        const uint32_t x = pixel % (uint32_t)cam.W, y = pixel / (uint32_t)cam.W;
        s.out = idx;
        s.pixel = pixel;
        rng.key = lgpu_path_key(rp.seed, pixel, sidx);
        rng.dim = 0;
        if (NS == 4) {
            const float u = lgpu_rng_float(rng.key, LGPU_DIM_WAVELENGTH);
            const float l0 = 380.0f + HERO_RANGE * u;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float l = l0 + (float)k * (HERO_RANGE / 4.0f);
                if (l >= 720.0f) l -= HERO_RANGE;
                lam.l[k] = l;
            }
        }
        camera_ray(cam, W.S.fpool, x, y, rng, s.ro, s.rd);
        s.L = Spec<NS>(0.f);
        s.beta = Spec<NS>(1.f);
        s.hit.tFar = finf(); s.hit.uv = make_float2(0.f, 0.f);
        s.ev.wo = -s.rd; s.ev.wi = mk(0.f, 0.f, 0.f); s.ev.woL = s.ev.wi; s.ev.wiL = s.ev.wi;
        s.ev.sidedness = 1; s.ev.medium = -1; s.ev.eta = 1.001f; s.ev.mediumInteraction = false;
        s.scatterIntersect = 0;
        s.nullCrossings = 0;
        s.bounces = 0;
        s.pc = PC_LOOP;
    }

    /* Run the state machine until the path issues a query or ends. */
    __device__ void run() {
        const DeviceScene &S = W.S;
        const RenderParams &rp = W.views ? W.views[s.view].rp : W.rp;
        const int maxB = rp.max_bounces, minB = rp.min_bounces;
#ifdef LGPU_STATE_CLOCKS
        StateClock clk(W.counters ? W.counters + 4 : nullptr);
#endif
        for (int guard = 0; guard < 4096; ++guard) {
#ifdef LGPU_STATE_CLOCKS
            clk.tick(s.pc);
#endif
            switch (s.pc) {
            case PC_LOOP: {
                if (s.bounces >= maxB) { s.pc = PC_DONE; break; }
                if (s.bounces == 0) { issue(s.ro, s.rd, finf(), Q_CLOSEST, PC_TOP_HIT); return; }
                s.pc = s.scatterIntersect ? PC_BODY : PC_MISS;
                break;
            }
            case PC_TOP_HIT: {
                HitRec hr;
                const bool ok = closest(hr);
                if (ok) process_hit(S, s.ro, s.rd, hr, s.hit);
                s.pc = ok ? PC_BODY : PC_MISS;
                break;
            }
            case PC_MISS: {
                if (s.bounces == 0 && S.env_light >= 0) s.L += T().env_le(s.rd) * s.beta;
                s.pc = PC_DONE;
                break;
            }
            case PC_BODY: {
                auto t = T();
                if (s.bounces == 0) {
                    const int li = t.mat(s.hit).light;
                    if (li >= 0) {
                        LRef lr; lr.light = li; lr.tri = -1;
                        if (s.ev.medium >= 0) s.L += t.light_L(lr, s.ev, s.hit) * medium_tr<NS>(S.media[s.ev.medium], s.hit.tFar);
                        else s.L += t.light_L(lr, s.ev, s.hit);
                    }
                }
                if (s.ev.medium >= 0) s.pc = PC_MED_A;
                else { s.ev.mediumInteraction = false; s.pc = PC_SURF_A; }
                break;
            }
            case PC_SURF_A: {
                auto t = T();
                const DMaterial &m = t.mat(s.hit);
                if (m.has_bsdf) {
                    s.ev.wo = -s.rd;
                    s.ev.woL = ev_local(s.hit, s.ev.wo);
                    s.ev.wiL = ev_local(s.hit, s.ev.wi);
                    s.ev.sidedness = (s.ev.woL.y > 0.f) ? 1 : -1;
                    s.lightDistPdf = 1.f;
                    s.sp = s.hit.point; s.sn = s.hit.nS;
                    float ldp = 1.f;
                    s.l = t.sample_light(s.hit.point, s.hit.nS, &ldp);
                    s.lightDistPdf = ldp;
                    if (li_prepare()) return;
                    s.visOK = 0;
                    s.visMode = -1;
                    s.pc = PC_SURF_LI;
                } else {
                    s.ev.medium = t.get_medium(m, s.rd, s.hit.nG);
                    s.ro = s.hit.point + s.hit.nG * (dot(s.hit.nG, s.rd) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
                    if (s.bounces > 0) { issue(s.ro, s.rd, finf(), Q_CLOSEST, PC_NULL_EXT); return; }
                    if (++s.nullCrossings > 256) { s.pc = PC_DONE; break; }
                    s.bounces--;
                    s.pc = PC_NEXT_ITER;
                }
                break;
            }
            case PC_NULL_EXT: {
                HitRec hr;
                const bool ok = closest(hr);
                if (ok) process_hit(S, s.ro, s.rd, hr, s.hit);
                s.scatterIntersect = ok;
                if (++s.nullCrossings > 256) { s.pc = PC_DONE; break; }
                s.bounces--;
                s.pc = PC_NEXT_ITER;
                break;
            }
            case PC_SURF_LI: {
                auto t = T();
                const DMaterial &m = t.mat(s.hit);
                const Spec<NS> Li = s.visMode >= 0 ? li_complete() : Spec<NS>(0.f);
                s.lightPDF *= s.lightDistPdf;
                Bsdf<NS> b;
                t.setup_bsdf(b, m, s.ev, s.hit);
                Spec<NS> Ld(0.f), f;
                float scatteringPDF = 0.f;
                if (s.lightPDF > 0.f && !Li.black()) {
                    f = bsdf_f<NS>(b, s.ev) * fabsf(s.ev.wiL.y);
                    scatteringPDF = bsdf_pdf<NS>(b, s.ev.woL, s.ev.wiL);
                    if (!f.black() && scatteringPDF > 0.f) {
                        const float w = Tracer<NS, COUNT>::power_heuristic(s.lightPDF, scatteringPDF);
                        Ld += Li * f * w / s.lightPDF;
                    }
                }
                f = bsdf_sample<NS>(b, s.ev, s.hit, rng, scatteringPDF);
                f *= fabsf(s.ev.wiL.y);
                s.ro = s.hit.point;
                s.rd = s.ev.wi;
                s.ev.medium = t.get_medium(m, s.ev.wi, s.hit.nG);
                s.Ld = Ld; s.f = f; s.scatteringPDF = scatteringPDF;
                if (scatteringPDF > 0.f && !f.black()) { issue(s.ro, s.rd, finf(), Q_CLOSEST, PC_SURF_EXT); return; }
                s.pc = PC_DONE;   /* `else break;` -- the NEE term of this vertex is dropped as in the reference */
                break;
            }
            case PC_SURF_EXT: {
                auto t = T();
                HitRec hr;
                const bool ok = closest(hr);
                if (ok) process_hit(S, s.ro, s.rd, hr, s.hit);
                s.scatterIntersect = ok;
                LRef nl; nl.light = ok ? t.mat(s.hit).light : S.env_light; nl.tri = -1;
                Spec<NS> Ld = s.Ld;
                if (nl.light >= 0) {
                    float ldp = s.lightDistPdf;
                    if (!lref_eq(nl, s.l)) ldp = t.light_pdf(s.sp, s.sn, s.hit.prim, nl);
                    const float lightPDF = ldp * t.pdf_li(nl, s.ev, s.hit);
                    const Spec<NS> Li = ok ? t.light_L(nl, s.ev, s.hit) : t.light_Le(nl, s.rd);
                    const float w = Tracer<NS, COUNT>::power_heuristic(s.scatteringPDF, lightPDF);
                    if (!Li.black() && lightPDF > 0.f) Ld += Li * s.f * w / s.scatteringPDF;
                }
                s.L += s.beta * Ld;
                s.beta *= s.f / s.scatteringPDF;
                s.pc = PC_RR;
                break;
            }
            case PC_RR: {
                if (s.bounces > minB) {
                    const float q = smax(.05f, 1.f - spec_y<NS>(s.beta, lam));
                    if (rng.next() < q) { s.pc = PC_DONE; break; }
                    s.beta /= 1.f - q;
                }
                s.pc = PC_NEXT_ITER;
                break;
            }
            case PC_NEXT_ITER: {
                s.bounces++;
                s.pc = PC_LOOP;
                break;
            }
            case PC_MED_A: {
                auto t = T();
                const DMedium &med = S.media[s.ev.medium];
                c.mPdf = 1.f;
                s.sp = s.hit.point; s.sn = s.hit.nS;
                float mp = 1.f;
                c.ml = t.sample_light(s.hit.point, s.hit.nS, &mp);
                float3 lp, ln = mk(0.f, 0.f, 0.f);
                c.mLe = t.sample_point(c.ml, s.ev, s.hit, lp, ln, mp);
                c.mPdf = mp; c.mPoint = lp; c.mNormal = ln;
                c.choice = (rng.next() > 0.5f) ? 0 : 1;
                float distT, distPdf, eqT, eqPdf;
                c.mTrD = medium_sample_distance<NS>(med, rng, s.ev, s.hit, &distT, &distPdf);
                const bool intD = s.ev.mediumInteraction;
                c.mTrE = medium_sample_equiangular<NS>(med, s.ro, s.rd, rng, s.ev, s.hit, c.mPoint, &eqT, &eqPdf);
                const bool intE = s.ev.mediumInteraction;
                s.ev.mediumInteraction = intD && intE;
                if (!s.ev.mediumInteraction) { s.beta *= c.mTrD; s.pc = PC_SURF_A; break; }
                s.ev.wo = -s.rd;
                c.mLd = Spec<NS>(0.f);
                c.mpD = s.ro + s.rd * distT;
                c.mpE = s.ro + s.rd * eqT;
                const float distPdf2 = medium_pdf_distance<NS>(med, eqT);
                const float eqPdf2 = medium_pdf_equiangular(s.ro, s.rd, c.mPoint, s.hit.tFar, distT);
                c.distW = Tracer<NS, COUNT>::power_heuristic(distPdf, eqPdf2);
                c.eqW = Tracer<NS, COUNT>::power_heuristic(eqPdf, distPdf2);
                c.medK = 0;
                s.pc = PC_LDM_START;
                break;
            }
            case PC_LDM_START: {
                const float3 p = c.medK == 0 ? c.mpD : c.mpE;
                c.kPartial = c.mPdf;
                s.hit.point = p;
                ldm_vis_prepare(p);
                if (s.pc != PC_LDM_VIS) return;   /* a query was issued */
                break;
            }
            case PC_LDM_VIS: {
                auto t = T();
                const DMedium &med = S.media[s.ev.medium];
                const float3 p = c.medK == 0 ? c.mpD : c.mpE;
                const Spec<NS> Li = c.mLe * ldm_vis_complete(p);
                const float lightPDF = c.mPdf;
                Spec<NS> kLd(0.f);
                if (lightPDF > 0.f && !Li.black()) {
                    const float sp = phase_hg(dot(s.ev.wo, s.ev.wi), med.g);
                    if (sp > 0.f) {
                        const float w = Tracer<NS, COUNT>::power_heuristic(lightPDF, sp);
                        kLd += Li * Spec<NS>(sp) * w / lightPDF;
                    }
                }
                c.kLd = kLd;
                float3 wi;
                c.kPhasePdf = hg_sample(med.g, s.ev.wo, &wi, rng);
                s.ev.wi = wi;
                if (c.medK == 0) c.wiD = wi; else c.wiE = wi;
                start_tr(p, wi, s.ev.medium, TR_EVENT, -1.f, PC_LDM_SCAT);
                return;
            }
            case PC_LDM_SCAT: {
                auto t = T();
                const bool hs = s.trResult != 0;
                const Spec<NS> Tr = s.trTr;
                Spec<NS> kLd = c.kLd;
                if (c.kPhasePdf > 0.f) {
                    LRef nl; nl.light = hs ? t.mat(s.hit).light : S.env_light; nl.tri = -1;
                    if (nl.light >= 0) {
                        if (!lref_eq(nl, c.ml)) c.kPartial = t.light_pdf(s.sp, s.sn, s.hit.prim, nl);
                        const float lightPDF = c.kPartial * t.pdf_li(nl, s.ev, s.hit);
                        const Spec<NS> Li = hs ? t.light_L(nl, s.ev, s.hit) : t.light_Le(nl, s.ev.wi);
                        const float w = Tracer<NS, COUNT>::power_heuristic(c.kPhasePdf, lightPDF);
                        if (!Li.black() && lightPDF > 0.f) kLd += Li * Tr * w / c.kPhasePdf;
                    }
                }
                if (c.medK == 0) { c.mLd += kLd * c.mTrD * c.distW; c.medK = 1; s.pc = PC_LDM_START; break; }
                c.mLd += kLd * c.mTrE * c.eqW;
                s.ro = c.choice == 0 ? c.mpD : c.mpE;
                s.rd = c.choice == 0 ? c.wiD : c.wiE;
                issue(s.ro, s.rd, finf(), Q_CLOSEST, PC_MED_EXT);
                return;
            }
            case PC_MED_EXT: {
                HitRec hr;
                const bool ok = closest(hr);
                if (ok) process_hit(S, s.ro, s.rd, hr, s.hit);
                s.scatterIntersect = ok;
                s.L += c.mLd;
                s.beta *= (c.choice == 0 ? c.mTrD : c.mTrE);
                s.pc = PC_RR;
                break;
            }
            case PC_VIS_OCCL: {
                s.visOK = occluded() ? 0 : 1;
                s.trTr = Spec<NS>(1.f);
                s.pc = s.visRet;
                break;
            }
            case PC_VIS_TR: {
                if (s.visMode == VIS_ESCAPE) s.visOK = s.trResult ? 0 : 1;
                else s.visOK = s.tmpTFar > s.visM - SURFACE_EPSILON * 10.f;
                s.pc = s.visRet;
                break;
            }
            case PC_TR_STEP: {   /* one segment of Scene::IntersectTr (Scene.cpp:45-81) */
                auto t = T();
                HitRec hr;
                if (NS == 3 && W.fold_tr) {
                    /* the trace kernel ran the whole walk: the state its last step leaves */
                    const float4 a = W.tr_out[2 * slot], b = W.tr_out[2 * slot + 1];
                    const int fl = __float_as_int(b.w);
                    s.trTr = Spec<NS>::from4(a);
                    c.trTFar = a.w;
                    s.trResult = fl & 1;
                    if (fl & 2) {
                        closest(hr);
                        const float fin = (fl & 1) ? c.trTFar : hr.t;   /* h.tFar the last step left */
                        if (c.trTarget == TR_EVENT) {
                            process_hit(S, mk(b.x, b.y, b.z), c.trD, hr, s.hit);
                            s.hit.tFar = fin;
                        } else {
                            s.tmpTFar = fin;
                        }
                    }
                    s.pc = c.trRet;
                    break;
                }
                if (!closest(hr)) { s.trResult = 0; s.pc = c.trRet; break; }
                RayHit tmp;
                RayHit &h = c.trTarget == TR_EVENT ? s.hit : tmp;
                process_hit(S, c.trO, c.trD, hr, h);
                if (c.trTarget == TR_TEMP) s.tmpTFar = h.tFar;
                c.trTFar += h.tFar;
                bool term = false;
                if (c.trMaxT >= 0.f) {
                    term = c.trTFar > c.trMaxT;
                    if (term) { const float delta = c.trTFar - c.trMaxT; c.trTFar -= delta; h.tFar -= delta; }
                }
                if (c.trMed >= 0) s.trTr *= medium_tr<NS>(S.media[c.trMed], h.tFar);
                const DMaterial &m = t.mat(h);
                if (term || m.has_bsdf || m.light >= 0) {
                    h.tFar = c.trTFar;
                    if (c.trTarget == TR_TEMP) s.tmpTFar = c.trTFar;
                    s.trResult = 1;
                    s.pc = c.trRet;
                    break;
                }
                c.trMed = t.get_medium(m, c.trD, h.nG);
                c.trO = h.point + h.nG * (dot(h.nG, c.trD) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
                if (++c.trIter >= 256) { s.trResult = 0; s.pc = c.trRet; break; }
                issue(c.trO, c.trD, finf(), Q_CLOSEST, PC_TR_STEP);
                return;
            }
            case PC_DONE:
            default:
                return;
            }
        }
    }
};

}  // namespace lg
