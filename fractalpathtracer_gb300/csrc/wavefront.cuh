// wavefront.cuh -- wavefront path tracer: persistent march kernel + shade kernel.
//
// renderPath (shaders/Shaders.metal:5926-6026) is split at its marches.  A
// wave of paths (pixel, sample) lives in device memory as PathRec records;
// work moves through queues of path indices:
//
//   camera_kernel   writes every path's camera ray into the march queue
//   march_kernel    persistent: each lane takes one march job (a path ray or
//                   a sun shadow ray) from the queue, marches it with one
//                   distance evaluation per loop iteration, and once it has
//                   finished takes the next job together with the warp's
//                   other finished lanes (per-lane regeneration in groups, one
//                   warp-aggregated atomic per refill); hits go to the shade
//                   queue, misses add the environment
//   shade_kernel    material, normal, sun shadow ray, scatter and Russian
//                   roulette of every hit; continuing paths go back to the
//                   march queue
//   finalize_kernel combines each path's light into its sample colour
//
// The sun term of a bounce only adds light (the scatter does not depend on
// it), so shadow rays of bounce b march in the same pass as the path rays of
// bounce b+1.  Random numbers are keyed by (pixel, sample, bounce), so the
// order in which work is scheduled never changes a path.
#pragma once

#include "fpt_march.cuh"
#include "fpt_kernels.h"

namespace fpt {

// PF_ESCAPED: the surrogate-skip pass found the ray leaving the geometry's
// box; the march classifies it as a miss without evaluating.  PF_KNOWN_D:
// the skip pass handed the ray over with the exact distance at its position
// in grad.w, so the march does not evaluate it again.
// PF_FP64: the camera ray's hit came from the FP64 continuation; its FP64
// distance from the camera is grad.w + shadow.w (high and low floats).
enum PathFlags : uint32_t {
    PF_DONE = 1u << 8, PF_INVISIBLE = 1u << 9, PF_VALID = 1u << 10, PF_ESCAPED = 1u << 11, PF_KNOWN_D = 1u << 12,
    PF_FP64 = 1u << 13
};

struct alignas(16) PathRec {
    float4 pos;     // xyz march origin or hit point, w side
    float4 dir;     // xyz direction, w sky mask
    float4 color;   // xyz throughput, w state bits (bounce | flags)
    float4 light;   // xyz emission + environment light, w slot bits
    float4 shadow;  // xyz sun light from shadow rays, w plain-march steps a camera ray took before the march kernel
    float4 grad;    // xyz background gradient colour of the camera ray, w exact distance (PF_KNOWN_D)
};
static_assert(sizeof(PathRec) == 96, "path records are six float4");

// A camera ray that enters the surrogate's box, queued by the camera kernel
// for the skip pass.
struct alignas(16) SkipJob {
    float4 origin;  // xyz march start of the camera ray, w path index bits
    float4 dir;     // xyz direction, w plain-march steps already taken (0 or 1)
};

struct alignas(16) ShadowJob {
    float4 origin;  // xyz hit point, w path index bits
    float4 normal;  // xyz normal the ray leaves along (offset 0.001), w advance made by the skip pass
    float4 dir;     // xyz light direction, w 1 when the skip pass found the ray leaving the geometry's box,
                    // 2 when it handed the ray over with the exact distance at its start in contrib.w
    float4 contrib; // xyz light added when the ray escapes
};

// Device counters of one wave.
enum Counter : uint32_t { C_MARCH0 = 0, C_MARCH1 = 1, C_SHADOW0 = 2, C_SHADOW1 = 3, C_SHADE = 4, C_HEAD = 5, C_SKIP = 6, C_SKIPN = 7,
                          C_COUNT = 8 };
// Word after the wave counters (not cleared between waves): set when a
// persistent loop ran past its time limit and gave up (the host reports it).
constexpr uint32_t C_GUARD = 8;
// Word holding the plain march's first step from a pinhole camera (float
// bits; written by first_step_kernel, read by the camera kernel).
constexpr uint32_t C_CAMSTEP = 9;
// Profile counters (FptSdfProfileStats): 0-2 march steps of primary /
// secondary / shadow rays, 3 normal evaluations, 4 bounces, 5 finished paths,
// 7 material evaluations, 8-10 orbit iterations of primary / secondary /
// shadow rays, 11 refinement steps, 12 most steps of one march, 13 most
// march steps of one path (all its rays: max_pixel_steps), 14 orbit
// iterations of normal evaluations.
constexpr int kProfileSlots = 16;
// Lockstep march: finished lanes write their results and take new rays in
// groups of this many (measured at 1080p 16 spp: 2 -> 863, 4 -> 923, 8 -> 944,
// 16 -> 903 Mpaths/s, against 797 when every lane refills at once).
constexpr uint32_t kRefillBatch = 8;
constexpr unsigned long long kLoopLimitNs = 10000000000ull;   // 10 s; a pass takes milliseconds

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Every 1024 trips: true (for the whole warp) once the loop has run past the
// limit; the first lane to see it records the error.
__device__ __forceinline__ bool loop_guard(uint32_t &trips, unsigned long long t0, uint32_t *counters, unsigned long long limit_ns) {
    if ((++trips & 1023u) != 0u) return false;
    const bool over = global_ns() - t0 > limit_ns;
    if (!__any_sync(0xffffffffu, over)) return false;
    if ((threadIdx.x & 31u) == 0u) atomicOr(counters + C_GUARD, 1u);
    return true;
}

// The scene of a single-scene launch, copied into this translation unit's
// constant memory before the launch (scene_to_constant): all lanes read the
// same scene fields, which the constant cache serves as instruction operands
// instead of one load instruction per field and lane.
static __constant__ DeviceScene c_scene;
static inline cudaError_t scene_to_constant(const DeviceScene *scene, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(c_scene, scene, sizeof(DeviceScene), 0, cudaMemcpyDeviceToDevice, st);
}

struct WaveParams {
    const DeviceScene *scene;
    PathRec *paths;
    uint32_t *q_march[2];
    ShadowJob *q_shadow[2];
    uint32_t *q_shade;
    uint32_t *counters;
    float4 *sample_rgb;
    uint32_t wave_base;        // first work index of this wave
    uint32_t n_paths;          // paths in this wave
    uint32_t pixel_work;       // tiles * 32
    uint32_t tiles_x;
    uint32_t sample_begin, sample_count;
    unsigned long long *profile;   // kProfileSlots counters or null
    uint32_t *path_steps;          // profile renders: march steps of each path of the wave (all its rays), or null
    // Box holding all geometry (surrogate modes): a march starts where its
    // ray enters the box and ends as a miss where it leaves it.
    uint32_t box_on;
    float box_lo[3], box_hi[3];
    // Surrogate-skip pass: the camera kernel flags camera rays that miss the
    // box as escaped and queues the others here (count in C_SKIPN).
    uint32_t skip_queue;
    SkipJob *q_skip;
    // Batched scenes (multi-scene passes, one sample per pass; null otherwise).
    // A path's scene is bits 16..31 of its state word.
    const DeviceScene *scenes;
    const uint32_t *work_base;   // n_scenes + 1 entries: first work index of each scene
    const uint32_t *pixel_base;  // n_scenes + 1 entries: first pixel of each scene in accum / sample_rgb
    uint32_t n_scenes;
    const uint32_t *pass;        // sample index of the pass (device word, advanced by the pass graph)
    uint32_t refill_batch;       // lockstep march: finished lanes wait for this many (0: kRefillBatch, 1: none)
    unsigned long long loop_limit_ns;   // time limit of the persistent loops (guard word bit 1 when reached)
};

// Scene of work index g: the largest k with base[k] <= g (base[0] = 0).
__device__ __forceinline__ uint32_t batch_scene(const uint32_t *base, uint32_t n, uint32_t g) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= g) lo = mid; else hi = mid;
    }
    return lo;
}

// Forward slab test against the wave's box: [tn, tf] with tn >= 0.
__device__ __forceinline__ bool wave_box_span(const WaveParams &W, float3 p, float3 d, float &tn, float &tf) {
    tn = 0.0f;
    tf = 3.0e38f;
    const float pv[3] = {p.x, p.y, p.z}, dv[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dv[a] != 0.0f) {
            const float inv = 1.0f / dv[a];
            const float t0 = (W.box_lo[a] - pv[a]) * inv, t1 = (W.box_hi[a] - pv[a]) * inv;
            tn = fmaxf(tn, fminf(t0, t1));
            tf = fminf(tf, fmaxf(t0, t1));
        } else if (pv[a] < W.box_lo[a] || pv[a] > W.box_hi[a]) {
            return false;
        }
    }
    return tf >= tn;
}

__device__ __forceinline__ uint32_t fbits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ float bitsf(uint32_t v) { return __uint_as_float(v); }

// Warp-aggregated append: one atomic per warp for all participating lanes.
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool want) {
    unsigned mask = __activemask();
    unsigned bal = __ballot_sync(mask, want);
    if (!want) return 0xffffffffu;
    uint32_t lane = threadIdx.x & 31u;
    uint32_t leader = __ffs(bal) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(bal));
    base = __shfl_sync(bal, base, leader);
    return base + __popc(bal & ((1u << lane) - 1u));
}

// Appends the lanes of a whole BLOCK-thread block that want a slot in either
// of two queues, with one atomic per queue and block (the camera and shade
// kernels append millions of rays per pass; one atomic per warp on one
// counter serialises over a million warps).  Every thread of the block calls
// it.
constexpr uint32_t kCameraBlock = 256;
template <uint32_t BLOCK>
__device__ __forceinline__ void block_append2(uint32_t *counter0, bool want0, uint32_t &slot0, uint32_t *counter1, bool want1,
                                              uint32_t &slot1) {
    constexpr uint32_t kWarps = BLOCK / 32u;
    __shared__ uint32_t s_off[2][kWarps + 1];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const unsigned b0 = __ballot_sync(0xffffffffu, want0), b1 = __ballot_sync(0xffffffffu, want1);
    if (lane == 0) {
        s_off[0][warp] = uint32_t(__popc(b0));
        s_off[1][warp] = uint32_t(__popc(b1));
    }
    __syncthreads();
    if (threadIdx.x < 2u) {   // thread q: exclusive offsets of the warps, then the block's base in queue q
        uint32_t sum = 0;
        for (uint32_t w = 0; w < kWarps; ++w) {
            const uint32_t c = s_off[threadIdx.x][w];
            s_off[threadIdx.x][w] = sum;
            sum += c;
        }
        s_off[threadIdx.x][kWarps] = sum ? atomicAdd(threadIdx.x == 0 ? counter0 : counter1, sum) : 0u;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
    slot0 = s_off[0][kWarps] + s_off[0][warp] + uint32_t(__popc(b0 & below));
    slot1 = s_off[1][kWarps] + s_off[1][warp] + uint32_t(__popc(b1 & below));
    __syncthreads();   // s_off is reused by the next call
}

__device__ __forceinline__ void wave_pixel(const WaveParams &W, uint32_t path, uint32_t width, uint32_t height, uint32_t &px,
                                           uint32_t &py, uint32_t &s_rel, bool &valid) {
    uint32_t g = W.wave_base + path;
    s_rel = g / W.pixel_work;
    uint32_t idx = g - s_rel * W.pixel_work;
    uint32_t tile = idx >> 5, within = idx & 31u;
    uint32_t tx = tile % W.tiles_x, ty = tile / W.tiles_x;
    px = tx * 8u + (within & 7u);
    py = ty * 4u + (within >> 3);
    valid = px < width && py < height;
}

__device__ __forceinline__ PathRng path_rng(const DeviceScene &S, uint32_t pixel, uint32_t sample) {
    PathRng r;
    uint32_t px = pixel % S.width, py = pixel / S.width;
    float2 uv = screen_uv(px, py, S);
    r.init(S.rng == FPT_CUDA_RNG_PCG, S.seed, pixel, sample, uv.x, uv.y);
    return r;
}

// ---------------------------------------------------------------- camera
// The plain march's first step from a pinhole camera.  Every camera ray
// starts at the camera, so its first distance evaluation is the same for all
// of them.  With the box clip, camera rays start at this step: the clipped
// march then visits the plain march's positions, and the box only decides
// misses (rays that never meet it, or whose first step passes it) and exits.
// (A start at the box entry instead changes the positions the march visits,
// and where the distance estimate exceeds the true distance, as the
// Mandelbox's does seen from outside, the plain march's steps pass over
// surface that a march from the box entry finds.)  0 when the camera has a
// lens (origins differ) or the plain march ends at the camera; camera rays
// then start at the box entry.
template <int KIND>
__global__ void first_step_kernel(const DeviceScene *scene, uint32_t *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const DeviceScene &S = *scene;
    float s1 = 0.0f;
    if (!(S.camera_dof > 0.0f)) {
        const float3 cam = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
        const float d = scene_eval<KIND>(S, cam, EV_MAP).d;
        if (isfinite(d)) {
            if (S.sdf_id == FPT_SDF_MANDELBULBER) {   // march_update, Mandelbulber branch
                const float th = mandel_threshold(cam, S);
                if (!(d < th)) s1 = mandel_march_step(d, th, S);
            } else {                                  // march_update, FPT rule (lod = min_dist at the start)
                const float o = fabsf(d) * 0.99f;
                if (!(o < S.render[3]) && !(S.render[4] < o)) s1 = o;
            }
        }
    }
    *out = fbits(s1);
}

template <bool BATCH>
__global__ void __launch_bounds__(kCameraBlock) camera_kernel(WaveParams W) {
    // The warp's 32 consecutive path records are assembled here and leave as
    // 16-byte stores that cover its 3 KB of records contiguously.
    __shared__ PathRec s_rec[kCameraBlock];
    const uint32_t lane = threadIdx.x & 31u, wbase = threadIdx.x & ~31u;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p - threadIdx.x < W.n_paths; p += gridDim.x * blockDim.x) {
        bool in_wave = p < W.n_paths;
        uint32_t px = 0, py = 0, s_rel = 0, k = 0;
        bool valid = false;
        const DeviceScene *sp = BATCH ? W.scene : &c_scene;
        if (in_wave) {
            if (BATCH) {
                const uint32_t g = W.wave_base + p;
                k = batch_scene(W.work_base, W.n_scenes, g);
                sp = W.scenes + k;
                const uint32_t idx = g - W.work_base[k], tiles_x = (sp->width + 7u) / 8u;
                const uint32_t tile = idx >> 5, within = idx & 31u;
                px = (tile % tiles_x) * 8u + (within & 7u);
                py = (tile / tiles_x) * 4u + (within >> 3);
                valid = px < sp->width && py < sp->height;
            } else {
                wave_pixel(W, p, sp->width, sp->height, px, py, s_rel, valid);
            }
        }
        const DeviceScene &S = *sp;
        bool march = false, skip = false;
        float3 rp = mk3(0.0f), dr = mk3(0.0f, 0.0f, 1.0f);
        float steps0 = 0.0f;   // plain-march steps taken by the start (the skip queue's dir.w)
        if (valid) {
            uint32_t pixel = py * S.width + px;
            uint32_t sample = BATCH ? *W.pass : W.sample_begin + s_rel;
            float2 uv = screen_uv(px, py, S);
            PathRng rng;
            rng.init(S.rng == FPT_CUDA_RNG_PCG, S.seed, pixel, sample, uv.x, uv.y);
            PathRec R;
            // the path's colour slot: sample-major, so a warp's 8 x 4 tile writes whole rows of pixels
            uint32_t slot = BATCH ? W.pixel_base[k] + pixel : s_rel * (S.width * S.height) + pixel;
            R.light = make_float4(0.f, 0.f, 0.f, bitsf(slot));
            R.shadow = make_float4(0.f, 0.f, 0.f, 0.f);
            if (!camera_ray(S, uv, rng, true, rp, dr)) {
                R.color = make_float4(0.f, 0.f, 0.f, bitsf(PF_VALID | PF_DONE | PF_INVISIBLE | (k << 16)));
                R.pos = make_float4(0.f, 0.f, 0.f, 1.f);
                R.dir = make_float4(0.f, 0.f, 1.f, 0.f);
                R.grad = make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                bool done = S.bounces == 0u;
                R.pos = make_float4(rp.x, rp.y, rp.z, 1.0f);
                R.dir = make_float4(dr.x, dr.y, dr.z, 0.0f);
                R.color = make_float4(1.f, 1.f, 1.f, bitsf(PF_VALID | (done ? PF_DONE : 0u) | (k << 16)));
                float3 g = background_gradient(dr, S);
                R.grad = make_float4(g.x, g.y, g.z, 0.f);
                march = !done;
                if (march && W.box_on) {   // start at the plain march's first step (else the box entry)
                    float tn, tf;
                    if (!wave_box_span(W, rp, dr, tn, tf)) {
                        R.color.w = bitsf(fbits(R.color.w) | PF_ESCAPED);
                    } else {
                        const float s1 = bitsf(W.counters[C_CAMSTEP]);
                        const float t0 = s1 > 0.0f ? s1 : tn;
                        if (t0 > tf) {   // the plain march's first step passes the whole box
                            R.color.w = bitsf(fbits(R.color.w) | PF_ESCAPED);
                        } else {
                            if (t0 > 0.0f) {
                                rp = rp + dr * t0;
                                R.pos = make_float4(rp.x, rp.y, rp.z, 1.0f);
                            }
                            steps0 = s1 > 0.0f ? 1.0f : 0.0f;   // the plain march's first step is taken
                            R.shadow.w = steps0;
                            skip = W.skip_queue != 0u;
                        }
                    }
                }
            }
            s_rec[threadIdx.x] = R;
        } else {
            PathRec R;   // not a pixel of the image (state word 0)
            R.pos = R.dir = R.color = R.light = R.shadow = R.grad = make_float4(0.f, 0.f, 0.f, 0.f);
            s_rec[threadIdx.x] = R;
        }
        __syncwarp();
        {
            const float4 *src = reinterpret_cast<const float4 *>(s_rec + wbase);
            float4 *dst = reinterpret_cast<float4 *>(W.paths + (p - lane));
            const uint32_t records = min(32u, W.n_paths > p - lane ? W.n_paths - (p - lane) : 0u);
#pragma unroll
            for (uint32_t c = lane; c < 32u * 6u; c += 32u)
                if (c / 6u < records) dst[c] = src[c];
        }
        __syncwarp();
        uint32_t at = 0, sat = 0;
        block_append2<kCameraBlock>(&W.counters[C_MARCH0], march, at, &W.counters[C_SKIPN], skip, sat);
        if (march) W.q_march[0][at] = p;
        if (skip) {
            W.q_skip[sat].origin = make_float4(rp.x, rp.y, rp.z, bitsf(p));
            W.q_skip[sat].dir = make_float4(dr.x, dr.y, dr.z, steps0);
        }
    }
}

// ---------------------------------------------------------------- march
struct MarchJob {
    uint32_t path;      // path index
    uint32_t bounce;
    bool shadow;
    float4 contrib;     // shadow: light to add when unoccluded
    float3 rp0;         // shadow: hit point the ray leaves
};

// FP64: the camera-ray pass of a deep-zoom scene (FptCudaSceneExt.fp64_bisection,
// a pinhole camera): a camera ray whose FP32 march stopped because a step no
// longer moved its position (shaders/Shaders.metal:3726, 3739-3746) continues
// in FP64 (march_fp64), which decides hit or miss and the hit distance.
template <int KIND, bool BATCH = false, int BLOCK = 128, int MINB = 7, bool FP64 = false>
__global__ void __launch_bounds__(BLOCK, MINB) march_kernel(WaveParams W, int cur) {
    const DeviceScene *sp = BATCH ? W.scene : &c_scene;   // the lane's scene (per job when BATCH)
    const uint32_t n_path = W.counters[C_MARCH0 + cur];
    const uint32_t total = n_path + W.counters[C_SHADOW0 + cur];
    const uint32_t *qm = W.q_march[cur];
    const ShadowJob *qs = W.q_shadow[cur];
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned FULL = 0xffffffffu;
    float3 cam = BATCH ? mk3(0.0f) : mk3(sp->cam_pos[0], sp->cam_pos[1], sp->cam_pos[2]);
    March m;
    MarchJob job;
    float3 box_origin = mk3(0.0f);   // box mode: ray origin and exit advance of the lane's job
    float box_exit = 3.0e38f;
    float known_d = 0.0f;            // exact distance at the march start handed over by the skip pass
    bool have_d = false;
    bool active = false, pending = false, retired = false;
    uint32_t c_primary = 0, c_secondary = 0, c_shadow = 0, c_paths = 0;
    // Profile counters kept off the registers of the march: orbit iterations of
    // the lane's current job in one register, block totals in shared memory
    // (updated when a march finishes, flushed at the end).
    __shared__ unsigned int s_prof[5];   // orbit iterations primary / secondary / shadow, refinement steps, longest march
    __shared__ unsigned int s_warps_done;
    uint32_t c_job_orbit = 0;
    if (W.profile) {   // the same in every thread
        if (threadIdx.x < 5) s_prof[threadIdx.x] = 0u;
        if (threadIdx.x == 0) s_warps_done = 0u;
        __syncthreads();
    }
    uint32_t trips = 0;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (loop_guard(trips, t0, W.counters, W.loop_limit_ns)) break;
        // Refill every lane whose march finished: one atomic per warp.
        unsigned need = __ballot_sync(FULL, !active && !pending && !retired);
        if (need) {
            uint32_t leader = __ffs(need) - 1, base = 0;
            if (lane == leader) base = atomicAdd(&W.counters[C_HEAD], (unsigned)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (!active && !pending && !retired) {
                uint32_t idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx >= total) {
                    retired = true;
                } else if (idx < n_path) {
                    job.path = qm[idx];
                    job.shadow = false;
                    const PathRec &R = W.paths[job.path];
                    float4 pos = R.pos, dir = R.dir;
                    uint32_t st = fbits(R.color.w);
                    if (BATCH) {
                        sp = W.scenes + (st >> 16);
                        cam = mk3(sp->cam_pos[0], sp->cam_pos[1], sp->cam_pos[2]);
                    }
                    const DeviceScene &S = *sp;
                    job.bounce = st & 0xffu;
                    int ni = job.bounce == 0u ? int(S.render[1]) : int(S.render[1] / (S.render[5] * 2.0f + 1.0f));
                    float3 o = mk3(pos.x, pos.y, pos.z), dv = mk3(dir.x, dir.y, dir.z);
                    float tn = 0.0f, tf = 3.0e38f;
                    if (W.box_on && !(st & PF_ESCAPED) && !wave_box_span(W, o, dv, tn, tf)) st |= PF_ESCAPED;
                    if (st & PF_ESCAPED) {   // a miss: end beyond the far limit
                        active = false;
                        m.steps = 0;
                        m.pos = o + dv * (S.render[4] + len3(o - cam) + 1.0f);
                    } else {
                        box_origin = o;
                        // Leaving the box ends camera rays as misses (their march would end beyond the far limit from
                        // the camera).  Later path rays keep marching: the reference counts a bounce whose march stops
                        // within the far limit of the camera as a hit (shaders/Shaders.metal:5971-5976), wherever it
                        // stops, and the box must not change that.
                        box_exit = job.bounce == 0u ? tf : 3.0e38f;
                        // the camera kernel (or the skip pass) placed camera rays; later rays start inside the box
                        const int before = job.bounce == 0u ? int(R.shadow.w) : 0;
                        if (before > 0)   // resumes the plain march from the camera (first step s1, or the skip pass's)
                            active = march_resume(m, S, cam, o, dv, ni, S.render[3], 0.0002f, before,
                                                  before == 1 ? bitsf(W.counters[C_CAMSTEP]) : 0.0f);
                        else
                            active = march_begin(m, S, o, dv, ni, S.render[3], 0.0002f);
                        have_d = active && (st & PF_KNOWN_D);
                        known_d = R.grad.w;
                    }
                    pending = !active;
                } else {
                    const ShadowJob &J = qs[idx - n_path];
                    float4 o = J.origin, nn = J.normal, d = J.dir;
                    job.path = fbits(o.w);
                    job.shadow = true;
                    if (BATCH) {
                        sp = W.scenes + (fbits(W.paths[job.path].color.w) >> 16);
                        cam = mk3(sp->cam_pos[0], sp->cam_pos[1], sp->cam_pos[2]);
                    }
                    const DeviceScene &S = *sp;
                    job.contrib = J.contrib;
                    job.rp0 = mk3(o.x, o.y, o.z);
                    float3 dv = mk3(d.x, d.y, d.z);
                    float3 start = job.rp0 + mk3(nn.x, nn.y, nn.z) * 0.001f + dv * nn.w;
                    float tn = 0.0f, tf = 3.0e38f;
                    const bool miss = d.w == 1.0f || (W.box_on && !wave_box_span(W, start, dv, tn, tf));
                    if (miss) {   // unoccluded: end beyond the far limit
                        active = false;
                        m.steps = 0;
                        m.pos = job.rp0 + dv * (S.render[4] * 1.01f + 1.0f);
                    } else {
                        box_origin = start;
                        box_exit = tf;
                        active = march_begin(m, S, start, dv, int(S.render[1]), S.render[3], 0.0002f);
                        have_d = active && d.w == 2.0f;
                        known_d = J.contrib.w;
                    }
                    pending = !active;
                }
            }
        }
        if (!__any_sync(FULL, !retired)) break;
        const DeviceScene &S = *sp;
        TranslucencyProbe<KIND> probe{sp};
        // One distance evaluation for every lane with a march in flight.
        if (active) {
            const Eval ev = have_d ? Eval{known_d, 0.0f, 0, 0} : scene_eval<KIND>(S, m.pos, EV_MAP);
            const float d = ev.d;
            c_job_orbit += uint32_t(ev.iters);
            have_d = false;
            active = march_update(m, S, d, probe);
            if (active && W.box_on && dot(m.pos - box_origin, m.dir) > box_exit) {
                // left the box: nothing more to hit; end beyond the far limit (a miss / unoccluded)
                active = false;
                m.pos = job.shadow ? job.rp0 + m.dir * (S.render[4] * 1.01f + 1.0f)
                                   : m.pos + m.dir * (S.render[4] + len3(m.pos - cam) + 1.0f);
            }
            pending = !active;
        }
        // Finished lanes write their results (and are refilled on the next
        // trip) together once `refill_batch` of them wait or nothing else runs:
        // the divergent finish and refill code then runs on many lanes at once
        // instead of on one or two lanes nearly every trip.
        bool finish = pending;
        const uint32_t refill_batch = W.refill_batch ? W.refill_batch : kRefillBatch;
        if (refill_batch > 1u) {
            // both votes are taken by every lane (never inside a short-circuited expression)
            const unsigned pb = __ballot_sync(FULL, pending);
            const bool any_active = __any_sync(FULL, active);
            finish = pending && (uint32_t(__popc(pb)) >= refill_batch || !any_active);
        }
        if (finish) {
            pending = false;
            if (W.profile) {
                atomicAdd(&s_prof[job.shadow ? 2 : (job.bounce == 0u ? 0 : 1)], c_job_orbit);
                if (m.refine) atomicAdd(&s_prof[3], uint32_t(m.refine));
                atomicMax(&s_prof[4], uint32_t(m.steps));
            }
            c_job_orbit = 0;
            if (W.path_steps) atomicAdd(W.path_steps + job.path, uint32_t(m.steps));
            if (job.shadow) {
                c_shadow += m.steps;
                if (len3(job.rp0 - m.pos) > S.render[4] * 0.99f) {
                    float4 &sh = W.paths[job.path].shadow;
                    sh = make_float4(sh.x + job.contrib.x, sh.y + job.contrib.y, sh.z + job.contrib.z, sh.w);
                }
            } else {
                if (job.bounce == 0u) c_primary += m.steps; else c_secondary += m.steps;
                PathRec &R = W.paths[job.path];
                if (FP64 && job.bounce == 0u && m.stalled) {
                    // restart a few FP32 ulps before the stop (the FP32 position is only that accurate)
                    const float back = 8.0f * 1.1920929e-7f * fmaxf(fmaxf(fabsf(m.pos.x), fabsf(m.pos.y)), fmaxf(fabsf(m.pos.z), 1.0f));
                    double t64 = 0.0;
                    int st = 0;
                    const double t0 = fmax(double(len3(m.pos - box_origin)) - double(back), 0.0);
                    if (march_fp64<KIND>(S, box_origin, m.dir, t0, int(S.render[1]), t64, st)) {
                        m.pos = box_origin + normalize3(m.dir) * float(t64);
                        const float hi = float(t64);
                        R.grad.w = hi;
                        R.shadow.w = float(t64 - double(hi));
                        R.color.w = bitsf(fbits(R.color.w) | PF_FP64);
                    } else {
                        m.pos = m.pos + m.dir * (S.render[4] + len3(m.pos - cam) + 1.0f);   // no surface: a miss
                    }
                    c_primary += uint32_t(st);
                }
                float3 r = m.pos - cam;
                float travel2 = dot(r, r);
                float maxd = S.render[4], far = maxd * 0.99f;
                bool hit = !(travel2 > far * far);
                if (job.bounce == 0u && travel2 > maxd * maxd) R.dir.w = 1.0f;
                if (!hit) {
                    float4 dir = R.dir;
                    float3 env = environment(mk3(dir.x, dir.y, dir.z), S);
                    float4 col = R.color, li = R.light;
                    if (S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX) env = env * mk3(col.x, col.y, col.z);
                    R.light = make_float4(li.x + env.x, li.y + env.y, li.z + env.z, li.w);
                    R.color.w = bitsf(fbits(col.w) | PF_DONE);
                    c_paths += 1;
                } else {
                    R.pos = make_float4(m.pos.x, m.pos.y, m.pos.z, R.pos.w);
                }
                uint32_t at = warp_append(&W.counters[C_SHADE], hit);
                if (hit) W.q_shade[at] = job.path;
            }
        }
    }
    if (W.profile) {
        uint32_t v[4] = {c_primary, c_secondary, c_shadow, c_paths};
        const int slot[4] = {0, 1, 2, 5};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint32_t s = v[k];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
            if (lane == 0 && s) atomicAdd(W.profile + slot[k], (unsigned long long)s);
        }
    }
    if (W.profile) {
        // The block's last warp to leave the loop flushes the shared totals (no
        // block barrier: finished warps do not wait for the others).
        __threadfence_block();
        uint32_t last = 0;
        if (lane == 0) last = atomicAdd(&s_warps_done, 1u) == blockDim.x / 32u - 1u ? 1u : 0u;
        last = __shfl_sync(FULL, last, 0);
        if (last) {
            __threadfence_block();
            if (lane < 5) {
                const unsigned long long s = atomicAdd(&s_prof[lane], 0u);   // read after the other warps' updates
                if (lane < 4) {
                    if (s) atomicAdd(W.profile + 8 + lane, s);
                } else if (s) {
                    atomicMax(W.profile + 12, s);
                }
            }
        }
    }
}

// ---------------------------------------------------------------- shade
// Lambert + GGX lobe (Heitz 2014 height-correlated Smith masking, Schlick
// Fresnel): f_cos = BRDF * cos(theta_l) and the pdf of the 1/2-1/2 mixture.
__device__ __forceinline__ void ggx_eval(const DeviceScene &S, float3 n, float3 v, float3 l, float albedo, bool plane,
                                         float3 &f_cos, float &pdf) {
    float nl = dot(n, l), nv = dot(n, v);
    if (nl <= 0.0f || nv <= 0.0f) { f_cos = mk3(0.0f); pdf = 0.0f; return; }
    float diffuse = albedo * (1.0f / kPi);
    if (plane) { f_cos = mk3(diffuse * nl); pdf = nl * (1.0f / kPi); return; }
    float a = S.ggx_alpha, a2 = a * a;
    float3 h = normalize3(v + l);
    float nh = dot(n, h);
    float dd = nh * nh * (a2 - 1.0f) + 1.0f;
    float D = a2 / (kPi * dd * dd);
    float tv = fmaxf(1.0f - nv * nv, 0.0f) / fmaxf(nv * nv, 1e-12f);
    float tl = fmaxf(1.0f - nl * nl, 0.0f) / fmaxf(nl * nl, 1e-12f);
    float lv = (sqrtf(1.0f + a2 * tv) - 1.0f) * 0.5f, ll = (sqrtf(1.0f + a2 * tl) - 1.0f) * 0.5f;
    float G = 1.0f / (1.0f + lv + ll);
    float F = S.specular_f0 + (1.0f - S.specular_f0) * pow5f(1.0f - fmaxf(dot(v, h), 0.0f));
    float spec = D * G * F / (4.0f * nv * nl);
    f_cos = mk3((diffuse * (1.0f - F) + spec) * nl);
    pdf = 0.5f * nl * (1.0f / kPi) + 0.5f * (1.0f / (1.0f + lv)) * D / (4.0f * nv);
}

template <int KIND, bool BATCH = false>
__global__ void __launch_bounds__(128) shade_kernel(WaveParams W, int cur) {
    const int next = cur ^ 1;
    const uint32_t n = W.counters[C_SHADE];
    uint32_t c_normal = 0, c_material = 0, c_paths = 0, c_bounces = 0, c_normal_orbit = 0;
    uint32_t *const normal_orbit = W.profile ? &c_normal_orbit : nullptr;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n; i += gridDim.x * blockDim.x) {
        bool live = i < n;
        bool emit_march = false, emit_shadow = false;
        uint32_t path = 0;
        ShadowJob J;
        if (live) {
            path = W.q_shade[i];
            PathRec R = W.paths[path];
            uint32_t state = fbits(R.color.w);
            const DeviceScene &S = BATCH ? W.scenes[state >> 16] : c_scene;
            const bool ggx = S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX;
            const int bounce = int(state & 0xffu);
            const uint32_t slot = fbits(R.light.w);
            uint32_t pixel, sample;
            if (BATCH) {
                pixel = slot - W.pixel_base[state >> 16];
                sample = *W.pass;
            } else {
                const uint32_t pixels = S.width * S.height;
                pixel = slot % pixels;
                sample = W.sample_begin + slot / pixels;
            }
            PathRng rng = path_rng(S, pixel, sample);
            float3 hit = mk3(R.pos.x, R.pos.y, R.pos.z), dr = mk3(R.dir.x, R.dir.y, R.dir.z);
            float3 color = mk3(R.color.x, R.color.y, R.color.z), light = mk3(R.light.x, R.light.y, R.light.z);
            float side = R.pos.w;
            // Material and normal (userSdf + normalAt, shaders/Shaders.metal:5980-5982).
            Material mt;
            float3 nrm;
            c_material += 1;
            if (bounce == 0 && (state & PF_FP64)) {
                // deep zoom: the normal at the FP64 hit point (the FP32 position is thresholds away from it)
                const double t64 = double(R.grad.w) + double(R.shadow.w);
                double dx = dr.x, dy = dr.y, dz = dr.z;
                const double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
                dx *= inv; dy *= inv; dz *= inv;
                nrm = normal_fp64<KIND>(S, double(S.cam_pos[0]) + dx * t64, double(S.cam_pos[1]) + dy * t64,
                                        double(S.cam_pos[2]) + dz * t64);
                mt = material_of(S, scene_eval<KIND>(S, hit, EV_MATERIAL));
                if (ggx) {
                    mt = default_material();
                    mt.rgb = mk3(S.albedo);
                    mt.surface = 0;
                }
                c_normal += 6;
            } else if (S.formula != 0 && S.ext_normal == FPT_CUDA_NORMAL_ANALYTIC && S.fractal_style_mode == 0u && ggx) {
                // One dual-number evaluation gives the surface id and the gradient.
                float3 g;
                analytic_gradient<KIND>(S, hit, g, normal_orbit);
                int surface = 0;
                if (S.ground_plane) {
                    Eval e = ext_eval<KIND>(S, hit);
                    surface = e.id;
                }
                mt = default_material();
                mt.rgb = mk3(surface ? S.plane_albedo : S.albedo);
                mt.surface = surface;
                nrm = (finite3(g) && dot(g, g) > 0.0f) ? normalize3(g) : mk3(0.f, 1.f, 0.f);
                c_normal += 1;
            } else {
                mt = material_of(S, scene_eval<KIND>(S, hit, EV_MATERIAL));
                nrm = normal_direct<KIND>(hit, S, normal_orbit);
                c_normal += normal_is_analytic(S) ? 1u : uint32_t(tap_count(S));
            }
            if (mt.emission > 0.001f) light = light + (ggx ? mt.rgb * (mt.emission) * color : mt.rgb * mt.emission);
            if (ggx && dot(nrm, dr) > 0.0f) nrm = -nrm;
            // Sun: direction with divergence, shadow ray (shaders/Shaders.metal:5846-5861).
            bool sun = S.sun[0] == 1.0f || (ggx && S.sun_power > 0.0f);
            if (sun) {
                float3 ld = mk3(S.sun_dir[0], S.sun_dir[1], S.sun_dir[2]);
                float h1 = rng.uniform(SLOT_SUN0, bounce), h2 = rng.uniform(SLOT_SUN1, bounce);
                float sa, ca;
                sincosf(h1 * 2.0f * kPi, &sa, &ca);
                float s = sqrtf(h2) * S.sun[4];
                ld = rotate_camera(ld, ca * s, sa * s);
                float3 contrib;
                float3 sc = mk3(S.sun_color[0], S.sun_color[1], S.sun_color[2]);
                if (ggx) {
                    float3 fc; float pdf;
                    ggx_eval(S, nrm, -dr, ld, mt.rgb.x, mt.surface == 1, fc, pdf);
                    float power = S.sun_power > 0.0f ? S.sun_power : S.sun[3];
                    contrib = fc * color * sc * power;
                    emit_shadow = dot(ld, nrm) > 0.0f;
                } else {
                    contrib = sc * (S.sun[3] * fmaxf(dot(nrm, ld), 0.0f) * mt.roughness * (1.0f - mt.translucency));
                    emit_shadow = true;
                }
                J.origin = make_float4(hit.x, hit.y, hit.z, bitsf(path));
                J.normal = make_float4(nrm.x, nrm.y, nrm.z, 0.f);
                J.dir = make_float4(ld.x, ld.y, ld.z, 0.f);
                J.contrib = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
            }
            // Scatter.
            bool terminate = false;
            if (ggx) {
                float3 v = -dr;
                float sgn = nrm.z >= 0.0f ? 1.0f : -1.0f;   // basis: Duff et al., JCGT 2017
                float aa = -1.0f / (sgn + nrm.z);
                float bb = nrm.x * nrm.y * aa;
                float3 t = mk3(1.0f + sgn * nrm.x * nrm.x * aa, sgn * bb, -sgn * nrm.x);
                float3 b = mk3(bb, sgn + nrm.y * nrm.y * aa, -nrm.y);
                float u1 = rng.uniform(SLOT_DIR0, bounce), u2 = rng.uniform(SLOT_DIR1, bounce);
                float3 l;
                if (mt.surface == 1 || rng.uniform(SLOT_LOBE, bounce) < 0.5f) {
                    float r = sqrtf(u1), sp, cp;
                    sincosf(2.0f * kPi * u2, &sp, &cp);
                    l = t * (r * cp) + b * (r * sp) + nrm * sqrtf(fmaxf(0.0f, 1.0f - u1));
                } else {
                    // Visible-normal sampling (Heitz, JCGT 2018).
                    float a = S.ggx_alpha;
                    float3 vl = mk3(dot(v, t), dot(v, b), dot(v, nrm));
                    float3 vh = normalize3(mk3(a * vl.x, a * vl.y, vl.z));
                    float lensq = vh.x * vh.x + vh.y * vh.y;
                    float3 t1 = lensq > 0.0f ? mk3(-vh.y, vh.x, 0.0f) * rsqrtf(lensq) : mk3(1.f, 0.f, 0.f);
                    float3 t2 = cross3(vh, t1);
                    float r = sqrtf(u1), sp, cp;
                    sincosf(2.0f * kPi * u2, &sp, &cp);
                    float p1 = r * cp, p2 = r * sp;
                    float sm = 0.5f * (1.0f + vh.z);
                    p2 = (1.0f - sm) * sqrtf(fmaxf(1.0f - p1 * p1, 0.0f)) + sm * p2;
                    float3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2));
                    float3 hl = normalize3(mk3(a * nh.x, a * nh.y, fmaxf(0.0f, nh.z)));
                    float3 h = t * hl.x + b * hl.y + nrm * hl.z;
                    l = reflect3(-v, h);
                }
                float3 fc; float pdf;
                ggx_eval(S, nrm, v, l, mt.rgb.x, mt.surface == 1, fc, pdf);
                if (!(pdf > 0.0f)) terminate = true;
                else {
                    color = color * (fc / pdf);
                    dr = normalize3(l);
                    hit = hit + nrm * (0.001f * signf(dot(dr, nrm)));
                }
            } else {
                float r1 = rng.uniform(SLOT_SCATTER, bounce), r2 = rng.uniform(SLOT_FRESNEL, bounce);
                float3 nn = nrm;
                if (r1 > mt.translucency) {
                    float3 metal = reflect3(dr, nn);
                    float h1 = rng.uniform(SLOT_DIR0, bounce), h2 = rng.uniform(SLOT_DIR1, bounce);   // randomVector :557-569
                    float3 nz = normalize3(nn);
                    float3 uu = normalize3(cross3(nz, mk3(0.0f, 1.0f, 1.0f)));
                    float3 vv = cross3(uu, nz);
                    float ra = sqrtf(h2), sr, cr;
                    sincosf(kPi * 2.0f * h1, &sr, &cr);
                    float3 diffuse = normalize3(uu * (ra * cr) + vv * (ra * sr) + nz * sqrtf(fmaxf(1.0f - h2, 0.0f)));
                    float f0 = (mt.ior - 1.0f) / (mt.ior + 1.0f);
                    f0 = f0 * f0;
                    float ct = clampf(dot(nn, -dr), 0.0f, 1.0f);
                    float fres = f0 + (1.0f - f0) * pow5f(1.0f - ct);
                    float3 ndir = normalize3(mix3(metal, diffuse, mt.roughness));
                    if (r2 < fres * mt.specular) ndir = metal;
                    else color = color * mt.rgb;
                    dr = ndir;
                } else {
                    float eta = side == 1.0f ? 1.0f / mt.ior : mt.ior;
                    if (side != 1.0f) nn = -nn;
                    float f0 = (mt.ior - 1.0f) / (mt.ior + 1.0f);
                    f0 = f0 * f0;
                    float ct = clampf(dot(nn, -dr), 0.0f, 1.0f);
                    float fres = f0 + (1.0f - f0) * pow5f(1.0f - ct);
                    float3 refr = refract3(dr, nn, eta);
                    float3 refl = reflect3(dr, nn);
                    if (dot(refr, refr) < 0.000001f || !isfinite(refr.x) || r2 < fres) {
                        dr = normalize3(refl);
                    } else {
                        dr = normalize3(refr);
                        side *= -1.0f;
                        color = color * (mix3(mk3(1.0f), mt.rgb, 0.35f) * (1.0f - fres * 0.5f));
                    }
                }
                hit = hit + nn * (0.001f * signf(dot(dr, nn)));
            }
            // Russian roulette (shaders/Shaders.metal:6016-6021).
            if (!terminate && S.russian_roulette != 0u && bounce + 1 < int(S.bounces) && float(bounce + 1) >= S.rr_start) {
                float surv = clampf(maxc3(color), clampf(S.rr_min_prob, 0.01f, 1.0f), 1.0f);
                if (rng.uniform(SLOT_RR, bounce) > surv) terminate = true;
                else color = color / surv;
            }
            if (!terminate && bounce + 1 >= int(S.bounces)) terminate = true;
            emit_march = !terminate;
            uint32_t nstate = (state & ~(0xffu | PF_KNOWN_D)) | uint32_t(bounce + 1) | (terminate ? PF_DONE : 0u);
            if (terminate) c_paths += 1;
            R.pos = make_float4(hit.x, hit.y, hit.z, side);
            R.dir = make_float4(dr.x, dr.y, dr.z, R.dir.w);
            R.color = make_float4(color.x, color.y, color.z, bitsf(nstate));
            R.light = make_float4(light.x, light.y, light.z, R.light.w);
            W.paths[path] = R;
        }
        c_bounces += emit_march ? 1u : 0u;
        uint32_t at = 0, sat = 0;
        block_append2<128>(&W.counters[C_MARCH0 + next], emit_march, at, &W.counters[C_SHADOW0 + next], emit_shadow, sat);
        if (emit_march) W.q_march[next][at] = path;
        if (emit_shadow) W.q_shadow[next][sat] = J;
    }
    if (W.profile) {
        uint32_t v[5] = {c_normal, c_material, c_paths, c_bounces, c_normal_orbit};
        const int slot[5] = {3, 7, 5, 4, 14};
        const unsigned FULL = 0xffffffffu;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            uint32_t s = v[k];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
            if ((threadIdx.x & 31u) == 0 && s) atomicAdd(W.profile + slot[k], (unsigned long long)s);
        }
    }
}

// One pass of a batch: accum = mix(accum, sample, 1 / (pass + 1)) over every
// pixel of every scene (the in-order mean of reduce_samples_kernel, one
// sample at a time), then the pass index advances for the next replay.
static __global__ void __launch_bounds__(256) reduce_pass_kernel(const float4 *sample_rgb, float4 *accum, uint32_t pixels,
                                                                 const uint32_t *pass) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pixels) return;
    const uint32_t i = *pass;
    float3 mean = mk3(0.0f);
    if (i > 0u) { const float4 a = accum[p]; mean = mk3(a.x, a.y, a.z); }
    const float4 c = sample_rgb[p];
    mean = mix3(mean, mk3(c.x, c.y, c.z), 1.0f / float(i + 1u));
    accum[p] = make_float4(mean.x, mean.y, mean.z, 1.0f);
}
static __global__ void advance_pass_kernel(uint32_t *pass) {
    if (threadIdx.x == 0) *pass += 1u;
}

// Resets the counters the next pass appends to.
static __global__ void reset_counters_kernel(uint32_t *counters, int next) {
    if (threadIdx.x == 0) {
        counters[C_MARCH0 + next] = 0u;
        counters[C_SHADOW0 + next] = 0u;
        counters[C_SHADE] = 0u;
        counters[C_HEAD] = 0u;
        counters[C_SKIP] = 0u;
    }
}

// Path colour: (light + sun light) times throughput (reference estimator)
// or the throughput-weighted sum (extension estimator), gradient mix and
// the 8.0 clamp of renderPath (shaders/Shaders.metal:6023-6025).
template <bool BATCH>
__global__ void __launch_bounds__(256) finalize_kernel(WaveParams W) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (W.path_steps) {   // profile renders: the largest march-step total of one path
        uint32_t v = p < W.n_paths ? W.path_steps[p] : 0u;
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((threadIdx.x & 31u) == 0u && v) atomicMax(W.profile + 13, (unsigned long long)v);
    }
    if (p >= W.n_paths) return;
    const PathRec &R = W.paths[p];
    uint32_t state = fbits(R.color.w);
    if (!(state & PF_VALID)) return;
    const DeviceScene &S = BATCH ? W.scenes[state >> 16] : c_scene;
    float3 col = mk3(0.0f);
    if (!(state & PF_INVISIBLE)) {
        float3 light = mk3(R.light.x + R.shadow.x, R.light.y + R.shadow.y, R.light.z + R.shadow.z);
        col = S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX ? light : light * mk3(R.color.x, R.color.y, R.color.z);
        if (S.world[6] == 1.0f) col = mix3(col, mk3(R.grad.x, R.grad.y, R.grad.z), R.dir.w);
        col = min3(col, mk3(8.0f));
    }
    W.sample_rgb[fbits(R.light.w)] = make_float4(col.x, col.y, col.z, 1.0f);
}

}  // namespace fpt
