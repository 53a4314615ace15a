/* Launch parameters shared by the API layer and the render kernels (internal). */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "lgpu_scene.h"

namespace lg {

struct CamParams {
    float3 o, x, y, z;
    float tanFov, tanFov2, aspect;
    float xi, yi;   /* 1 / width, 1 / height */
    int W, H;
    int type;       /* lgpu_camera_type */
    int aperture;   /* lgpu_aperture_type (thin lens) */
    int blades;
    float focal, ap_size, off_phi, off_theta;
    /* masked aperture: Piecewise2D of the mask in the scene's float pool (rows of 2w + 2 floats:
     * CDF, function, integral; then the marginal CDF and function) */
    int mask_cond_off, mask_marg_off, mask_w, mask_h;
    float mask_marg_int;
};
struct RenderParams {
    int spp, max_bounces, min_bounces;
    uint32_t seed, sample_offset;
    int integrator;   /* lgpu_integrator (megakernel only; the wavefront runs the MIS integrator) */
};
/* One view of a batched render: its camera and parameters, and the index of its first path within
 * the chunk of views being rendered (paths of a view are pixel-major, spp per pixel). */
struct DView {
    CamParams cam;
    RenderParams rp;
    uint64_t first;
};
struct LaunchArgs {
    DeviceScene S;
    CamParams cam;
    RenderParams rp;
    float4 *film;
    float4 *paths_out;
    const uint64_t *ids;
    uint64_t n;
    unsigned long long *counters;
    bool hero, count;
    cudaStream_t stream;
};

cudaError_t launch_render_3_0(const LaunchArgs &a);
cudaError_t launch_render_3_1(const LaunchArgs &a);
cudaError_t launch_render_4_0(const LaunchArgs &a);
cudaError_t launch_render_4_1(const LaunchArgs &a);
/* the integrators other than GPU_MISVOLPATH (launch_render_* forwards to these) */
cudaError_t launch_render_other_3_0(const LaunchArgs &a);
cudaError_t launch_render_other_3_1(const LaunchArgs &a);
cudaError_t launch_render_other_4_0(const LaunchArgs &a);
cudaError_t launch_render_other_4_1(const LaunchArgs &a);
inline cudaError_t launch_render(const LaunchArgs &a) {
    if (a.hero) return a.count ? launch_render_4_1(a) : launch_render_4_0(a);
    return a.count ? launch_render_3_1(a) : launch_render_3_0(a);
}
struct WaveArgs;
cudaError_t wave_resume_3_0(const WaveArgs &W, int n, int start_new, cudaStream_t st);
cudaError_t wave_resume_3_1(const WaveArgs &W, int n, int start_new, cudaStream_t st);
cudaError_t wave_resume_4_0(const WaveArgs &W, int n, int start_new, cudaStream_t st);
cudaError_t wave_resume_4_1(const WaveArgs &W, int n, int start_new, cudaStream_t st);
cudaError_t wave_trace_3_0(const WaveArgs &W, int n, cudaStream_t st, int block = 128);
cudaError_t wave_trace_3_1(const WaveArgs &W, int n, cudaStream_t st, int block = 128);
size_t wave_state_bytes_3_0();
size_t wave_cold_bytes_3_0();
size_t wave_cold_bytes_4_0();
size_t wave_cold_bytes_3_1();
size_t wave_cold_bytes_4_1();
size_t wave_state_bytes_4_0();
size_t wave_state_bytes_3_1();
size_t wave_state_bytes_4_1();
cudaError_t film_resolve(const float4 *film, float4 *rgba, uint64_t n_px, cudaStream_t st);
cudaError_t film_reduce(const float4 *paths, float4 *film, uint64_t first_px, uint64_t n_px, int spp, cudaStream_t st);
cudaError_t read_probe(const float4 *p, uint64_t n4, int passes, float *sink, int blocks, cudaStream_t st);
struct AdjArgs;
cudaError_t launch_adjoint(const DeviceScene &S, const CamParams &cam, const RenderParams &rp, const AdjArgs &A,
                           uint64_t n, cudaStream_t st);
cudaError_t launch_intersect(const DeviceScene &S, const float *rays, uint32_t *hits, float *uvs, uint64_t n, cudaStream_t s);

}  // namespace lg
