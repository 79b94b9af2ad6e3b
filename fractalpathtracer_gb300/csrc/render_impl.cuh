// render_impl.cuh -- sphere-tracing kernels for sm_103a (templated on the scene kind).
//
// Hot kernel: pathtrace_persistent<KIND>, a persistent megakernel in which
// every lane owns one pixel's path (renderPath, shaders/Shaders.metal:
// 5926-6026) as a resumable state machine.  Each warp iteration:
//   1. lanes that finished their pixel take new pixels from a global
//      counter with one warp-aggregated atomic (ray regeneration);
//   2. lanes post a request -- one distance evaluation at a point, or one
//      analytic normal;
//   3. the warp executes the request kind most lanes want (warp-level
//      compaction by operation), so the distance estimator runs with all
//      requesting lanes converged; analytic normals are batched until
//      enough lanes wait for one.
// Samples of a pixel run in order in one lane, so the running mean matches
// the reference's accumulate kernels (7706-7773) bit for bit in any
// accumulation mode.
#pragma once

#include "fpt_march.cuh"
#include "fpt_kernels.h"

namespace fpt {

// ---------------------------------------------------------------- path lane
enum LanePhase : uint8_t {
    LP_NEED_WORK = 0,
    LP_RETIRED = 1,
    LP_PATH_MARCH = 2,
    LP_MATERIAL = 3,
    LP_TAP = 4,
    LP_GRAD = 5,
    LP_SHADOW_MARCH = 6,
};
enum Request : uint8_t { RQ_NONE = 0, RQ_EVAL = 1, RQ_GRAD = 2 };

struct Lane {
    // work
    uint32_t pixel, sample, sample_end;
    float3 mean;
    float2 uv;
    PathRng rng;
    // path
    float3 dr, light, color, grad_col, hit, n, tap_acc, sun_dir;
    float side, sky_mask, eps;
    int bounce, local_ni, tap;
    Material mt;
    March m;
    // request
    uint8_t phase, req, mode;
    float3 q;
    // counters
    uint32_t c_primary, c_secondary, c_shadow, c_normal, c_bounces, c_evals, c_material, c_pixels;
};

struct PathParams {
    const DeviceScene *scene;
    float4 *accum;
    unsigned int *work_counter;
    uint32_t total_work;       // tiles * 32
    uint32_t tiles_x;          // 8-pixel-wide tiles per row
    uint32_t sample_begin, sample_end;
    uint32_t grad_batch;       // analytic normals run when this many lanes wait (or nothing else is pending)
    unsigned long long *profile;  // 8 counters or null
};

// Work index -> pixel: 8x4 tiles so a warp's 32 first pixels are adjacent.
__device__ __forceinline__ bool work_pixel(const PathParams &P, uint32_t idx, uint32_t W, uint32_t H, uint32_t &px, uint32_t &py) {
    uint32_t tile = idx >> 5, within = idx & 31u;
    uint32_t tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    px = tx * 8u + (within & 7u);
    py = ty * 4u + (within >> 3);
    return px < W && py < H;
}

template <int KIND> struct Path {
    const DeviceScene &S;
    TranslucencyProbe<KIND> probe;
    __device__ explicit Path(const DeviceScene &s) : S(s), probe{&s} {}

    __device__ void request_eval(Lane &L, float3 q, int mode) { L.req = RQ_EVAL; L.q = q; L.mode = uint8_t(mode); }
    __device__ void request_grad(Lane &L, float3 q) { L.req = RQ_GRAD; L.q = q; }

    // Starts the current sample of the lane's pixel; may finish it at once.
    __device__ void begin_sample(Lane &L) {
        L.rng.init(S.rng == FPT_CUDA_RNG_PCG, S.seed, L.pixel, L.sample, L.uv.x, L.uv.y);
        float3 rp;
        if (!camera_ray(S, L.uv, L.rng, true, rp, L.dr)) {
            finish_sample(L, mk3(0.0f));
            return;
        }
        L.side = 1.0f; L.light = mk3(0.0f); L.color = mk3(1.0f); L.sky_mask = 0.0f;
        L.grad_col = background_gradient(L.dr, S);
        L.bounce = 0;
        L.local_ni = int(S.render[1]);
        if (S.bounces == 0u) { end_path(L); return; }
        begin_path_march(L, rp);
    }

    __device__ void begin_path_march(Lane &L, float3 origin) {
        L.phase = LP_PATH_MARCH;
        if (march_begin(L.m, S, origin, L.dr, L.local_ni, S.render[3], 0.0002f)) request_eval(L, L.m.pos, EV_MAP);
        else path_march_done(L);
    }

    __device__ void path_march_done(Lane &L) {
        if (L.bounce == 0) L.c_primary += L.m.steps; else L.c_secondary += L.m.steps;
        L.c_evals += L.m.steps;
        float3 rp = L.m.pos;
        float3 cam = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
        float3 r = rp - cam;
        float travel2 = dot(r, r);
        float maxd = S.render[4], far = maxd * 0.99f;
        if (L.bounce == 0 && travel2 > maxd * maxd) L.sky_mask = 1.0f;
        L.local_ni = int(S.render[1] / (S.render[5] * 2.0f + 1.0f));
        L.c_bounces += 1;
        if (travel2 > far * far) {
            float3 env = environment(L.dr, S);
            L.light = L.light + (S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX ? env * L.color : env);
            end_path(L);
            return;
        }
        L.hit = rp;
        L.phase = LP_MATERIAL;
        request_eval(L, rp, EV_MATERIAL);
    }

    __device__ void material_done(Lane &L, const Eval &e) {
        L.c_material += 1; L.c_evals += 1;
        L.mt = material_of(S, e);
        if (S.brdf != FPT_CUDA_BRDF_LAMBERT_GGX && L.mt.emission > 0.001f) L.light = L.light + L.mt.rgb * L.mt.emission;
        if (S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX && L.mt.emission > 0.001f) L.light = L.light + L.mt.rgb * L.mt.emission * L.color;
        if (normal_is_analytic(S)) {
            L.phase = LP_GRAD;
            request_grad(L, L.hit);
        } else {
            begin_taps(L);
        }
    }

    __device__ void begin_taps(Lane &L) {
        L.phase = LP_TAP;
        L.tap = 0;
        L.tap_acc = mk3(0.0f);
        L.eps = normal_epsilon(L.hit, S);
        request_eval(L, L.hit + tap_offset(S, 0, L.eps), tap_mode(S));
    }

    __device__ void tap_done(Lane &L, float d) {
        L.c_normal += 1; L.c_evals += 1;
        tap_accumulate(S, L.tap, d, L.tap_acc);
        if (++L.tap < tap_count(S)) {
            request_eval(L, L.hit + tap_offset(S, L.tap, L.eps), tap_mode(S));
            return;
        }
        float3 acc = L.tap_acc;
        if (S.normal_mode != 1u && S.sdf_id == FPT_SDF_MANDELBULBER && !(fmaxf(fabsf(acc.x), fmaxf(fabsf(acc.y), fabsf(acc.z))) > 0.0f))
            acc = mandel_orbit_normal<KIND>(L.hit, L.eps, S);
        normal_done(L, normalize_fd(acc));
    }

    // Executes the analytic-normal request of a lane (batched across the warp).
    __device__ void run_grad(Lane &L) {
        L.c_normal += 1;
        if (S.sdf_id == FPT_SDF_MANDELBULBER && S.render[7] > 0.0f && !(S.formula != 0 && S.ext_normal == FPT_CUDA_NORMAL_ANALYTIC)) {
            normal_done(L, mandel_slow_normal<KIND>(L.hit, S));
            return;
        }
        float3 g;
        bool ok = analytic_gradient<KIND>(S, L.hit, g);
        if (S.formula != 0) {
            normal_done(L, (ok && finite3(g) && dot(g, g) > 0.0f) ? normalize3(g) : mk3(0.f, 1.f, 0.f));
            return;
        }
        if (ok) normal_done(L, normalize3(g));
        else begin_taps(L);   // invalid program gradient: fall back to finite differences
    }

    __device__ void normal_done(Lane &L, float3 n) {
        L.n = n;
        bool ggx = S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX;
        if (ggx && dot(L.n, L.dr) > 0.0f) L.n = -L.n;
        bool sun = S.sun[0] == 1.0f || (ggx && S.sun_power > 0.0f);
        if (sun) {
            // Sun direction with divergence (shaders/Shaders.metal:5846-5855).
            float3 ld = mk3(S.sun_dir[0], S.sun_dir[1], S.sun_dir[2]);
            float h1 = L.rng.uniform(SLOT_SUN0, L.bounce), h2 = L.rng.uniform(SLOT_SUN1, L.bounce);
            float sa, ca;
            sincosf(h1 * 2.0f * kPi, &sa, &ca);
            float s = sqrtf(h2) * S.sun[4];
            ld = rotate_camera(ld, ca * s, sa * s);
            L.sun_dir = ld;
            if (!ggx || dot(ld, L.n) > 0.0f) {
                L.phase = LP_SHADOW_MARCH;
                if (march_begin(L.m, S, L.hit + L.n * 0.001f, ld, int(S.render[1]), S.render[3], 0.0002f)) {
                    request_eval(L, L.m.pos, EV_MAP);
                } else {
                    shadow_done(L);
                }
                return;
            }
        }
        scatter(L);
    }

    __device__ void shadow_done(Lane &L) {
        L.c_shadow += L.m.steps; L.c_evals += L.m.steps;
        bool lit = len3(L.hit - L.m.pos) > S.render[4] * 0.99f;
        if (lit) {
            float3 sc = mk3(S.sun_color[0], S.sun_color[1], S.sun_color[2]);
            if (S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX) {
                float3 v = -L.dr;
                float3 fc; float pdf;
                brdf_eval(L, v, L.sun_dir, fc, pdf);
                float power = S.sun_power > 0.0f ? S.sun_power : S.sun[3];
                L.light = L.light + fc * L.color * sc * power;
            } else {
                L.light = L.light + sc * (S.sun[3] * fmaxf(dot(L.n, L.sun_dir), 0.0f) * L.mt.roughness * (1.0f - L.mt.translucency));
            }
        }
        scatter(L);
    }

    // Lambert + GGX lobe (Heitz 2014 height-correlated Smith masking,
    // Schlick Fresnel); f_cos = BRDF * cos(theta_l), pdf of the 1/2-1/2 mixture.
    __device__ void brdf_eval(const Lane &L, float3 v, float3 l, float3 &f_cos, float &pdf) {
        float3 n = L.n;
        float nl = dot(n, l), nv = dot(n, v);
        if (nl <= 0.0f || nv <= 0.0f) { f_cos = mk3(0.0f); pdf = 0.0f; return; }
        float albedo = L.mt.rgb.x;
        float diffuse = albedo * (1.0f / kPi);
        if (L.mt.surface == 1) { f_cos = mk3(diffuse * nl); pdf = nl * (1.0f / kPi); return; }
        float a = S.ggx_alpha, a2 = a * a;
        float3 h = normalize3(v + l);
        float nh = dot(n, h);
        float dd = nh * nh * (a2 - 1.0f) + 1.0f;
        float D = a2 / (kPi * dd * dd);
        auto lambda = [&](float c) {
            float c2 = c * c;
            float t2 = fmaxf(1.0f - c2, 0.0f) / fmaxf(c2, 1e-12f);
            return (sqrtf(1.0f + a2 * t2) - 1.0f) * 0.5f;
        };
        float lv = lambda(nv), ll = lambda(nl);
        float G = 1.0f / (1.0f + lv + ll);
        float F = S.specular_f0 + (1.0f - S.specular_f0) * pow5f(1.0f - fmaxf(dot(v, h), 0.0f));
        float spec = D * G * F / (4.0f * nv * nl);
        f_cos = mk3((diffuse * (1.0f - F) + spec) * nl);
        float pdf_spec = (1.0f / (1.0f + lv)) * D / (4.0f * nv);
        pdf = 0.5f * nl * (1.0f / kPi) + 0.5f * pdf_spec;
    }

    __device__ void scatter(Lane &L) {
        const int i = L.bounce;
        if (S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX) {
            float3 n = L.n, v = -L.dr;
            // Orthonormal basis: Duff et al., JCGT 2017.
            float sgn = n.z >= 0.0f ? 1.0f : -1.0f;
            float aa = -1.0f / (sgn + n.z);
            float bb = n.x * n.y * aa;
            float3 t = mk3(1.0f + sgn * n.x * n.x * aa, sgn * bb, -sgn * n.x);
            float3 b = mk3(bb, sgn + n.y * n.y * aa, -n.y);
            float u1 = L.rng.uniform(SLOT_DIR0, i), u2 = L.rng.uniform(SLOT_DIR1, i);
            float3 l;
            if (L.mt.surface == 1 || L.rng.uniform(SLOT_LOBE, i) < 0.5f) {
                float r = sqrtf(u1), sp, cp;
                sincosf(2.0f * kPi * u2, &sp, &cp);
                l = t * (r * cp) + b * (r * sp) + n * sqrtf(fmaxf(0.0f, 1.0f - u1));
            } else {
                // Visible-normal sampling (Heitz, JCGT 2018), local frame.
                float a = S.ggx_alpha;
                float3 vl = mk3(dot(v, t), dot(v, b), dot(v, n));
                float3 vh = normalize3(mk3(a * vl.x, a * vl.y, vl.z));
                float lensq = vh.x * vh.x + vh.y * vh.y;
                float3 t1 = lensq > 0.0f ? mk3(-vh.y, vh.x, 0.0f) * rsqrtf(lensq) : mk3(1.f, 0.f, 0.f);
                float3 t2 = cross3(vh, t1);
                float r = sqrtf(u1), sp, cp;
                sincosf(2.0f * kPi * u2, &sp, &cp);
                float p1 = r * cp, p2 = r * sp;
                float s = 0.5f * (1.0f + vh.z);
                p2 = (1.0f - s) * sqrtf(fmaxf(1.0f - p1 * p1, 0.0f)) + s * p2;
                float3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2));
                float3 hl = normalize3(mk3(a * nh.x, a * nh.y, fmaxf(0.0f, nh.z)));
                float3 h = t * hl.x + b * hl.y + n * hl.z;
                l = reflect3(-v, h);
            }
            float3 fc; float pdf;
            brdf_eval(L, v, l, fc, pdf);
            if (!(pdf > 0.0f)) { end_path(L); return; }
            L.color = L.color * (fc / pdf);
            L.dr = normalize3(l);
            L.hit = L.hit + n * (0.001f * signf(dot(L.dr, n)));
        } else {
            float3 n = L.n;
            float r1 = L.rng.uniform(SLOT_SCATTER, i), r2 = L.rng.uniform(SLOT_FRESNEL, i);
            const Material &mt = L.mt;
            if (r1 > mt.translucency) {
                float3 metal = reflect3(L.dr, n);
                // randomVector (shaders/Shaders.metal:557-569)
                float h1 = L.rng.uniform(SLOT_DIR0, i), h2 = L.rng.uniform(SLOT_DIR1, i);
                float3 nn = normalize3(n);
                float3 uu = normalize3(cross3(nn, mk3(0.0f, 1.0f, 1.0f)));
                float3 vv = cross3(uu, nn);
                float ra = sqrtf(h2), sr, cr;
                sincosf(kPi * 2.0f * h1, &sr, &cr);
                float3 diffuse = normalize3(uu * (ra * cr) + vv * (ra * sr) + nn * sqrtf(fmaxf(1.0f - h2, 0.0f)));
                float f0 = (mt.ior - 1.0f) / (mt.ior + 1.0f);
                f0 = f0 * f0;
                float ct = clampf(dot(n, -L.dr), 0.0f, 1.0f);
                float fres = f0 + (1.0f - f0) * pow5f(1.0f - ct);
                L.dr = normalize3(mix3(metal, diffuse, mt.roughness));
                if (r2 < fres * mt.specular) L.dr = metal;
                else L.color = L.color * mt.rgb;
            } else {
                float eta = L.side == 1.0f ? 1.0f / mt.ior : mt.ior;
                if (L.side != 1.0f) n = -n;
                float f0 = (mt.ior - 1.0f) / (mt.ior + 1.0f);
                f0 = f0 * f0;
                float ct = clampf(dot(n, -L.dr), 0.0f, 1.0f);
                float fres = f0 + (1.0f - f0) * pow5f(1.0f - ct);
                float3 refr = refract3(L.dr, n, eta);
                float3 refl = reflect3(L.dr, n);
                if (dot(refr, refr) < 0.000001f || !isfinite(refr.x) || r2 < fres) {
                    L.dr = normalize3(refl);
                } else {
                    L.dr = normalize3(refr);
                    L.side *= -1.0f;
                    L.color = L.color * (mix3(mk3(1.0f), mt.rgb, 0.35f) * (1.0f - fres * 0.5f));
                }
            }
            L.hit = L.hit + n * (0.001f * signf(dot(L.dr, n)));
        }
        // Russian roulette (shaders/Shaders.metal:6016-6021)
        if (S.russian_roulette != 0u && i + 1 < int(S.bounces) && float(i + 1) >= S.rr_start) {
            float surv = clampf(maxc3(L.color), clampf(S.rr_min_prob, 0.01f, 1.0f), 1.0f);
            float rr = L.rng.uniform(SLOT_RR, i);
            if (rr > surv) { end_path(L); return; }
            L.color = L.color / surv;
        }
        if (++L.bounce >= int(S.bounces)) { end_path(L); return; }
        begin_path_march(L, L.hit);
    }

    __device__ void end_path(Lane &L) {
        float3 col = S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX ? L.light : L.light * L.color;
        if (S.world[6] == 1.0f) col = mix3(col, L.grad_col, L.sky_mask);
        finish_sample(L, min3(col, mk3(8.0f)));
    }

    __device__ void finish_sample(Lane &L, float3 col) {
        L.mean = mix3(L.mean, col, 1.0f / float(L.sample + 1u));
        if (++L.sample < L.sample_end) {
            begin_sample(L);
            return;
        }
        L.req = RQ_NONE;
        L.phase = LP_NEED_WORK;
        L.c_pixels += 1;
    }

    // Consumes the result of the lane's RQ_EVAL request.
    __device__ void on_eval(Lane &L, const Eval &e) {
        switch (L.phase) {
            case LP_PATH_MARCH:
                if (march_update(L.m, S, e.d, probe)) request_eval(L, L.m.pos, EV_MAP);
                else path_march_done(L);
                break;
            case LP_SHADOW_MARCH:
                if (march_update(L.m, S, e.d, probe)) request_eval(L, L.m.pos, EV_MAP);
                else shadow_done(L);
                break;
            case LP_MATERIAL: material_done(L, e); break;
            case LP_TAP: tap_done(L, e.d); break;
            default: break;
        }
    }
};

template <int KIND>
__global__ void __launch_bounds__(128) pathtrace_persistent(PathParams P) {
    const DeviceScene &S = *P.scene;
    Path<KIND> path(S);
    const uint32_t lane_id = threadIdx.x & 31u;
    const unsigned FULL = 0xffffffffu;
    Lane L;
    L.phase = LP_NEED_WORK;
    L.req = RQ_NONE;
    L.c_primary = L.c_secondary = L.c_shadow = L.c_normal = L.c_bounces = L.c_evals = L.c_material = L.c_pixels = 0;
    const uint32_t W = S.width, H = S.height;
    uint32_t grad_wait = 0;   // warp iterations since a lane started waiting for an analytic normal
    while (true) {
        // 1. regeneration: one atomic per warp for every lane that needs work.
        unsigned need = __ballot_sync(FULL, L.phase == LP_NEED_WORK);
        if (need) {
            uint32_t leader = __ffs(need) - 1, base = 0;
            if (lane_id == leader) base = atomicAdd(P.work_counter, (unsigned)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (L.phase == LP_NEED_WORK) {
                uint32_t idx = base + __popc(need & ((1u << lane_id) - 1u));
                if (idx >= P.total_work) {
                    L.phase = LP_RETIRED;
                } else {
                    uint32_t px, py;
                    if (work_pixel(P, idx, W, H, px, py)) {
                        L.pixel = py * W + px;
                        L.uv = screen_uv(px, py, S);
                        L.sample = P.sample_begin;
                        L.sample_end = P.sample_end;
                        if (P.sample_begin == 0u) L.mean = mk3(0.0f);
                        else { float4 a = P.accum[L.pixel]; L.mean = mk3(a.x, a.y, a.z); }
                        if (L.sample < L.sample_end) path.begin_sample(L);
                        else { L.phase = LP_NEED_WORK; L.req = RQ_NONE; }
                        // finished without any request: write and ask again next round
                        if (L.phase == LP_NEED_WORK) P.accum[L.pixel] = make_float4(L.mean.x, L.mean.y, L.mean.z, 1.0f);
                    }
                    // pixels outside the image stay LP_NEED_WORK
                }
            }
        }
        unsigned alive = __ballot_sync(FULL, L.phase != LP_RETIRED);
        if (!alive) break;
        // 2. choose the operation of this iteration.
        unsigned want_eval = __ballot_sync(FULL, L.req == RQ_EVAL && L.phase >= LP_PATH_MARCH);
        unsigned want_grad = __ballot_sync(FULL, L.req == RQ_GRAD && L.phase >= LP_PATH_MARCH);
        grad_wait = want_grad ? grad_wait + 1u : 0u;
        bool do_grad = want_grad && (want_eval == 0u || (uint32_t)__popc(want_grad) >= P.grad_batch || grad_wait >= 24u);
        if (do_grad) grad_wait = 0u;
        // 3. execute it for the lanes that asked.
        if (!do_grad) {
            if (L.req == RQ_EVAL && L.phase >= LP_PATH_MARCH) {
                Eval e = scene_eval<KIND>(S, L.q, L.mode);
                path.on_eval(L, e);
                if (L.phase == LP_NEED_WORK) P.accum[L.pixel] = make_float4(L.mean.x, L.mean.y, L.mean.z, 1.0f);
            }
        } else if (L.req == RQ_GRAD && L.phase >= LP_PATH_MARCH) {
            path.run_grad(L);
            if (L.phase == LP_NEED_WORK) P.accum[L.pixel] = make_float4(L.mean.x, L.mean.y, L.mean.z, 1.0f);
        }
    }
    if (P.profile) {
        uint32_t v[8] = {L.c_primary, L.c_secondary, L.c_shadow, L.c_normal, L.c_bounces, L.c_pixels, L.c_evals, L.c_material};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            uint32_t s = v[k];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
            if (lane_id == 0) atomicAdd(P.profile + k, (unsigned long long)s);
        }
    }
}

// ---------------------------------------------------------------- primary rays
template <int KIND>
__global__ void __launch_bounds__(128) trace_primary_kernel(const DeviceScene *scene, FptCudaPrimaryHit *hits) {
    const DeviceScene &S = *scene;
    uint32_t gx = blockIdx.x * 16u + (threadIdx.x & 15u), gy = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (gx >= S.width || gy >= S.height) return;
    float2 uv = screen_uv(gx, gy, S);
    PathRng rng;
    rng.init(false, 0u, 0u, 0u, uv.x, uv.y);
    float3 rp, dr;
    FptCudaPrimaryHit h;
    h.distance = 0.0f; h.normal[0] = h.normal[1] = h.normal[2] = 0.0f; h.steps = 0; h.hit = 0;
    if (camera_ray(S, uv, rng, false, rp, dr)) {
        March m = march_loop<KIND>(S, rp, dr, int(S.render[1]), S.render[3], 0.0002f);
        float travel = len3(m.pos - rp);
        bool hit = m.found && isfinite(travel) && travel < S.render[4] * 0.99f;
        h.distance = travel;
        h.steps = uint32_t(m.steps);
        h.hit = hit ? 1u : 0u;
        if (hit) {
            float3 n = normal_direct<KIND>(m.pos, S);
            h.normal[0] = n.x; h.normal[1] = n.y; h.normal[2] = n.z;
        }
    }
    hits[size_t(gy) * S.width + gx] = h;
}

// ---------------------------------------------------------------- focus prepass
// estimate_focus_distance_kernel (shaders/Shaders.metal:5869-5884): one
// thread writes the resolved focus into the scene block in device memory.
template <int KIND>
__global__ void focus_kernel(DeviceScene *scene) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const DeviceScene &S = *scene;
    float3 cam = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
    float3 dr = rotate_camera(normalize3(mk3(0.0f, 0.0f, S.focal)), S.yaw, S.pitch, S.roll);
    March m = march_loop<KIND>(S, cam, dr, 120, 0.001f, 0.001f);
    float d = len3(m.pos - cam);
    if (!isfinite(d) || d <= 0.001f || d > S.render[4] * 0.99f) d = 5.0f;
    scene->focus_distance = d;
}

// ---------------------------------------------------------------- batch evaluation
// mandelbulber_field_sample_kernel (shaders/Shaders.metal:1001-1009).
template <int KIND>
__global__ void field_sample_kernel(const DeviceScene *scene, const float4 *points, float4 *samples, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = points[i];
    Field4 f = mandel_field<KIND>(mk3(p.x, p.y, p.z), *scene, 1);
    samples[i] = make_float4(f.d, f.r, f.dr, fabsf(f.state));
}

// distanceSdf (plus orbit, derivative, iterations where defined) and the
// analytic gradient at a batch of points.
template <int KIND>
__global__ void sample_distance_kernel(const DeviceScene *scene, const float4 *points, float4 *samples, float *grads, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DeviceScene &S = *scene;
    float4 p4 = points[i];
    float3 p = mk3(p4.x, p4.y, p4.z);
    Eval e = scene_eval<KIND>(S, p, EV_RAW);
    float dr = 0.0f, it = 0.0f;
    if (S.sdf_id == FPT_SDF_MANDELBULBER) {
        Field4 f = mandel_field<KIND>(p, S, 1);
        dr = f.dr; it = fabsf(f.state);
    }
    samples[i] = make_float4(e.d, S.formula ? e.orbit : 0.0f, dr, it);
    if (grads) {
        float3 g = mk3(0.0f);
        if (S.formula != 0 || S.sdf_id == FPT_SDF_PROGRAM) {
            if (!analytic_gradient<KIND>(S, p, g) && S.sdf_id == FPT_SDF_PROGRAM) g = program_gradient(p, S, nullptr);
        }
        grads[i * 3 + 0] = g.x; grads[i * 3 + 1] = g.y; grads[i * 3 + 2] = g.z;
    }
}

}  // namespace fpt
