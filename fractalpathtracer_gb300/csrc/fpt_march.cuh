// fpt_march.cuh -- sphere-tracing march as a resumable state machine.
//
// march_update() consumes one distance evaluation and either asks for the
// next one (returns true, evaluate at m.pos) or finishes.  The same code
// drives plain loops (primary rays, focus prepass) and the persistent path
// kernel, where every lane issues one evaluation per warp iteration.
#pragma once

#include "fpt_de.cuh"

namespace fpt {

struct March {
    float3 pos, dir, start;
    float th, step, dist, limit, min_dist, lod_falloff;
    int it, maxi, refine, steps;
    bool refining, found, done;
    bool stalled;   // ended because a step no longer changed the FP32 position
};

// sdfMarchIterationLimit: shaders/Shaders.metal:3626-3633
__device__ __forceinline__ int march_iteration_limit(int requested, const DeviceScene &S) {
    return min(requested, S.sdf_id == FPT_SDF_MANDELBULBER ? 10000 : 360);
}

// sdfMarchStep (Mandelbulber branch): shaders/Shaders.metal:3643-3681
__device__ __forceinline__ float mandel_march_step(float d, float th, const DeviceScene &S) {
    const float *v = S.vset_values;
    float step = fmaxf(d - 0.5f * th, 0.0f) * v[113];
    if (v[108] > 0.5f) {
        step = clampf(step, v[109], v[110]);
        if (th > v[109]) step = clampf(step, v[111] * th, v[112] * th);
    } else {
        step = fminf(step, v[110]);
    }
    return step;
}

__device__ __forceinline__ bool same3(float3 a, float3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Starts a march (march / marchMandelbulber, shaders/Shaders.metal:3700-3783).
// Returns true when an evaluation at m.pos is needed.
__device__ __forceinline__ bool march_begin(March &m, const DeviceScene &S, float3 origin, float3 dir, int ni, float min_dist,
                                            float lod_falloff) {
    m.pos = origin; m.dir = dir; m.start = origin;
    m.th = 0.0f; m.step = 0.0f; m.dist = 0.0f; m.limit = 1.0f;
    m.min_dist = min_dist; m.lod_falloff = lod_falloff;
    m.it = 0; m.maxi = march_iteration_limit(ni, S); m.refine = 0; m.steps = 0;
    m.refining = false; m.found = false; m.done = false; m.stalled = false;
    if (m.maxi <= 0) { m.done = true; return false; }
    return true;
}

__device__ __forceinline__ bool march_finish(March &m, bool found) { m.found = found; m.done = true; return false; }

// Resumes the march of a ray from `start` that has taken `it` steps, the
// last of length `step`, and stands at `pos`: the state march_update leaves
// there (the step budget and the distance limit count from `start`, a
// refinement starts from half of `step`).
__device__ __forceinline__ bool march_resume(March &m, const DeviceScene &S, float3 start, float3 pos, float3 dir, int ni, float min_dist,
                                             float lod_falloff, int it, float step) {
    const bool more = march_begin(m, S, pos, dir, ni, min_dist, lod_falloff);
    m.start = start;
    m.it = it;
    m.step = step;
    if (more && m.it >= m.maxi) return march_finish(m, false);
    return more;
}

// Mandelbulber refinement bracket: shaders/Shaders.metal:3733-3749.
__device__ __forceinline__ bool mandel_refine_move(March &m) {
    if (m.dist < m.th && m.dist > m.th * m.limit) return march_finish(m, true);
    if (m.dist > m.th) {
        float3 next = m.pos + m.dir * m.step;
        if (same3(next, m.pos)) { m.stalled = true; return march_finish(m, true); }
        m.pos = next;
    } else if (m.dist < m.th * m.limit) {
        float3 next = m.pos - m.dir * m.step;
        if (same3(next, m.pos)) { m.stalled = true; return march_finish(m, true); }
        m.pos = next;
    }
    return true;
}

// Consumes the distance d evaluated at m.pos (mapSdf).  `translucency_at`
// is only called for scenes with translucent materials (glass), as the
// reference does inside march().
template <class TranslucencyFn>
__device__ __forceinline__ bool march_update(March &m, const DeviceScene &S, float d, TranslucencyFn translucency_at) {
    ++m.steps;
    if (S.sdf_id == FPT_SDF_MANDELBULBER) {
        if (!m.refining) {
            m.th = mandel_threshold(m.pos, S);
            m.dist = d;
            if (!isfinite(d)) return march_finish(m, false);
            if (d < m.th) {
                m.limit = 1.0f - 0.001f * fmaxf(S.vset_values[129], 0.0f);
                m.step *= 0.5f;
                m.refine = 0;
                m.refining = true;
                return mandel_refine_move(m);
            }
            m.step = mandel_march_step(d, m.th, S);
            float3 next = m.pos + m.dir * m.step;
            if (same3(next, m.pos)) { m.stalled = true; return march_finish(m, false); }
            m.pos = next;
            if (len3(m.pos - m.start) >= S.render[4]) return march_finish(m, false);
            if (++m.it >= m.maxi) return march_finish(m, false);
            return true;
        }
        m.dist = d;
        m.step *= 0.5f;
        if (++m.refine >= 30) return march_finish(m, true);
        return mandel_refine_move(m);
    }
    // FPT rule: step 0.99|d|, converge when the step falls under the LOD
    // threshold, stop past render[4] (shaders/Shaders.metal:3753-3783).
    if (!isfinite(d)) return march_finish(m, false);
    float o = fabsf(d) * 0.99f;
    m.pos = m.pos + m.dir * o;
    float lod = m.min_dist;
    if (m.lod_falloff > 0.00001f) {
        float3 r = m.start - m.pos;
        float fog = dot(r, r);
        lod = mixf(lod, 0.1f, fog * m.lod_falloff);
        lod = mixf(m.min_dist, lod, S.render[5]);
    }
    if (S.translucent && translucency_at(m.pos) > 0.0f) lod = 0.0001f;
    if (o < lod) return march_finish(m, true);
    if (S.render[4] < o) return march_finish(m, false);
    if (++m.it >= m.maxi) return march_finish(m, false);
    return true;
}

template <int KIND> struct TranslucencyProbe {
    const DeviceScene *S;
    __device__ float operator()(float3 p) const {
        Eval e = scene_eval<KIND>(*S, p, EV_MATERIAL);
        return material_of(*S, e).translucency;
    }
};

// ---------------------------------------------------------------- FP64 continuation
// Deep-zoom cameras put the hit threshold below the FP32 resolution of the
// hit position: marchMandelbulber (shaders/Shaders.metal:3700-3751) then
// stops where a step no longer changes the position (3726) or where a
// refinement half-step does (3739-3746).  With DeviceScene::fp64_bisection
// the ray continues from there in FP64 -- positions along the ray and the
// extension orbit in double -- with the same step rule, threshold and
// 30-halving band search as the FP32 march.  Returns the hit distance from
// `origin` (false: no hit).
template <int KIND>
__device__ double de_fp64(const DeviceScene &S, double px, double py, double pz) {
    OrbitResult<double> o;
    switch (runtime_kind(KIND) ? S.kind : (uint32_t)KIND) {
        case KIND_BULB8: o = ext_field<KIND_BULB8, double>(S, px, py, pz, 1); break;
        case KIND_BULB: o = ext_field<KIND_BULB, double>(S, px, py, pz, 1); break;
        case KIND_BOX: o = ext_field<KIND_BOX, double>(S, px, py, pz, 1); break;
        case KIND_MENGER: o = ext_field<KIND_MENGER, double>(S, px, py, pz, 1); break;
        default: o = ext_field<KIND_HYBRID, double>(S, px, py, pz, 1); break;
    }
    return o.escaped ? o.d : -o.d;   // sign carries the escape state for mandel_finish
}

template <int KIND>
__device__ bool march_fp64(const DeviceScene &S, float3 origin, float3 dir, double t0, int max_steps, double &t_hit, int &steps) {
    const double ox = origin.x, oy = origin.y, oz = origin.z;
    double dx = dir.x, dy = dir.y, dz = dir.z;
    const double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
    dx *= inv; dy *= inv; dz *= inv;
    const double cx = S.cam_pos[0], cy = S.cam_pos[1], cz = S.cam_pos[2];
    const float *v = S.vset_values;
    auto eval = [&](double t, double &th) {
        const double px = ox + dx * t, py = oy + dy * t, pz = oz + dz * t;
        const double ex = px - cx, ey = py - cy, ez = pz - cz;
        th = v[115] > 0.5f ? sqrt(ex * ex + ey * ey + ez * ez) * double(v[116]) : double(v[117]);   // :3635-3641
        th = fmin(fmax(th, double(v[118])), double(v[119]));
        double signed_d = de_fp64<KIND>(S, px, py, pz);
        double d = fabs(signed_d);
        if (v[115] > 1.5f) {                                                                         // mandel_finish
            if (signed_d < 0.0) d = 0.0;
            else if (d < th) d = th * 1.01;
        }
        ++steps;
        return d + (d / 2.0 - d) * double(S.render[6]);
    };
    double t = t0, th = 0.0, step = 0.0;
    double dist = eval(t, th);
    bool found = false;
    for (int i = 0; i < max_steps && isfinite(dist); ++i) {
        if (dist < th) { found = true; break; }
        step = fmax(dist - 0.5 * th, 0.0) * double(v[113]);                                         // :3643-3681
        if (v[108] > 0.5f) {
            step = fmin(fmax(step, double(v[109])), double(v[110]));
            if (th > v[109]) step = fmin(fmax(step, double(v[111]) * th), double(v[112]) * th);
        } else {
            step = fmin(step, double(v[110]));
        }
        const double tn = t + step;
        if (tn == t || tn - t0 >= double(S.render[4])) break;
        t = tn;
        dist = eval(t, th);
    }
    if (!found) return false;
    const double limit = 1.0 - 0.001 * fmax(double(v[129]), 0.0);
    step *= 0.5;
    for (int r = 0; r < 30; ++r) {                                                                  // :3733-3749
        if (dist < th && dist > th * limit) break;
        if (dist > th) t += step;
        else if (dist < th * limit) t -= step;
        dist = eval(t, th);
        step *= 0.5;
    }
    t_hit = t;
    return true;
}

// Normal at an FP64 hit point: central differences of |DE| in FP64 with the
// normal epsilon of normalAt (the Mandelbulber threshold at the point times
// vset_values[114], shaders/Shaders.metal:3899-3901).  At deep zoom the FP32
// hit position is many thresholds from the surface, so a normal evaluated
// there would belong to other detail.
template <int KIND>
__device__ __noinline__ float3 normal_fp64(const DeviceScene &S, double px, double py, double pz) {
    const float *v = S.vset_values;
    const double ex = px - double(S.cam_pos[0]), ey = py - double(S.cam_pos[1]), ez = pz - double(S.cam_pos[2]);
    double th = v[115] > 0.5f ? sqrt(ex * ex + ey * ey + ez * ez) * double(v[116]) : double(v[117]);
    th = fmin(fmax(th, double(v[118])), double(v[119]));
    const double e = th * double(v[114]);
    const double gx = fabs(de_fp64<KIND>(S, px + e, py, pz)) - fabs(de_fp64<KIND>(S, px - e, py, pz));
    const double gy = fabs(de_fp64<KIND>(S, px, py + e, pz)) - fabs(de_fp64<KIND>(S, px, py - e, pz));
    const double gz = fabs(de_fp64<KIND>(S, px, py, pz + e)) - fabs(de_fp64<KIND>(S, px, py, pz - e));
    const double n = sqrt(gx * gx + gy * gy + gz * gz);
    if (!(n > 0.0) || !isfinite(n)) return mk3(0.0f, 1.0f, 0.0f);
    return mk3(float(gx / n), float(gy / n), float(gz / n));
}

// Plain-loop march (focus prepass, primary rays, diagnostics).
template <int KIND>
__device__ March march_loop(const DeviceScene &S, float3 origin, float3 dir, int ni, float min_dist, float lod_falloff) {
    March m;
    TranslucencyProbe<KIND> probe{&S};
    bool more = march_begin(m, S, origin, dir, ni, min_dist, lod_falloff);
    while (more) {
        float d = scene_eval<KIND>(S, m.pos, EV_MAP).d;
        more = march_update(m, S, d, probe);
    }
    return m;
}
// march_loop for a ray resumed at `pos` after `it` steps from `start` (march_resume).
template <int KIND>
__device__ March march_loop_from(const DeviceScene &S, float3 start, float3 pos, float3 dir, int ni, float min_dist, float lod_falloff,
                                 int it, float step) {
    March m;
    TranslucencyProbe<KIND> probe{&S};
    bool more = march_resume(m, S, start, pos, dir, ni, min_dist, lod_falloff, it, step);
    while (more) {
        float d = scene_eval<KIND>(S, m.pos, EV_MAP).d;
        more = march_update(m, S, d, probe);
    }
    return m;
}

// normalizeFiniteDifference: shaders/Shaders.metal:3863-3869
__device__ __forceinline__ float3 normalize_fd(float3 g) {
    float mm = fmaxf(fabsf(g.x), fmaxf(fabsf(g.y), fabsf(g.z)));
    if (!(mm > 0.0f) || !isfinite(mm)) return mk3(0.0f, 1.0f, 0.0f);
    return normalize3(g / mm);
}

// Normal epsilon of normalAt (shaders/Shaders.metal:3899-3901).
__device__ __forceinline__ float normal_epsilon(float3 p, const DeviceScene &S) {
    return S.sdf_id == FPT_SDF_MANDELBULBER ? mandel_threshold(p, S) * S.vset_values[114] : fmaxf(S.render[2], 0.0002f);
}
__device__ __forceinline__ int tap_count(const DeviceScene &S) { return S.normal_mode == 1u ? 4 : 6; }
// Offset of finite-difference tap k (central 6-tap or tetrahedral 4-tap).
__device__ __forceinline__ float3 tap_offset(const DeviceScene &S, int k, float e) {
    if (S.normal_mode == 1u) {
        float te = e * 0.57735026919f;
        float3 kk = k == 0 ? mk3(1.f, -1.f, -1.f) : (k == 1 ? mk3(-1.f, -1.f, 1.f) : (k == 2 ? mk3(-1.f, 1.f, -1.f) : mk3(1.f)));
        return kk * te;
    }
    float s = (k & 1) ? -e : e;
    return k < 2 ? mk3(s, 0.f, 0.f) : (k < 4 ? mk3(0.f, s, 0.f) : mk3(0.f, 0.f, s));
}
__device__ __forceinline__ void tap_accumulate(const DeviceScene &S, int k, float d, float3 &acc) {
    if (S.normal_mode == 1u) {
        float3 kk = k == 0 ? mk3(1.f, -1.f, -1.f) : (k == 1 ? mk3(-1.f, -1.f, 1.f) : (k == 2 ? mk3(-1.f, 1.f, -1.f) : mk3(1.f)));
        acc = acc + kk * d;
        return;
    }
    float s = (k & 1) ? -d : d;
    if (k < 2) acc.x += s; else if (k < 4) acc.y += s; else acc.z += s;
}
__device__ __forceinline__ int tap_mode(const DeviceScene &S) { return S.sdf_id == FPT_SDF_MANDELBULBER ? EV_NORMAL : EV_MAP; }

// Mandelbulber's slow-shading 11^3 iteration-field stencil (:3872-3896).
template <int KIND> __device__ float3 mandel_slow_normal(float3 p, const DeviceScene &S) {
    float delta = len3(mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]) - p) * S.render[7] * S.vset_values[114];
    float maxit = S.set_values[1];
    float3 sn = mk3(0.0f);
    for (int ix = -5; ix <= 5; ++ix)
        for (int iy = -5; iy <= 5; ++iy)
            for (int iz = -5; iz <= 5; ++iz) {
                float3 sd = mk3(float(ix), float(iy), float(iz)) * 0.2f;
                Field4 f = mandel_field<KIND>(p + sd * delta, S, 1);
                sn = sn + sd * (1.0f + maxit - fabsf(f.state));
            }
    float mm = fmaxf(fabsf(sn.x), fmaxf(fabsf(sn.y), fabsf(sn.z)));
    if (!(mm > 0.0f) || !isfinite(mm)) return mk3(1.0f, 0.0f, 0.0f);
    return normalize3(sn / mm);
}
// Orbit-radius fallback when every tap collapses (:3955-3969).
template <int KIND> __device__ float3 mandel_orbit_normal(float3 p, float e, const DeviceScene &S) {
    int mult = S.vset_values[115] > 1.5f ? 5 : 1;
    auto lr = [&](float3 q) { return logf(fmaxf(fabsf(mandel_field<KIND>(q, S, mult).r), 1.0e-30f)); };
    float3 xo = mk3(e, 0.f, 0.f), yo = mk3(0.f, e, 0.f), zo = mk3(0.f, 0.f, e);
    return mk3(lr(p + xo) - lr(p - xo), lr(p + yo) - lr(p - yo), lr(p + zo) - lr(p - zo));
}

// Does this scene take its normal from a single analytic request?
__device__ __forceinline__ bool normal_is_analytic(const DeviceScene &S) {
    if (S.formula != 0 && S.ext_normal == FPT_CUDA_NORMAL_ANALYTIC) return true;
    if (S.formula == 0 && S.sdf_id == FPT_SDF_PROGRAM && S.program_count > 0u && (S.normal_mode == 0u || S.normal_mode == 2u)) return true;
    if (S.sdf_id == FPT_SDF_MANDELBULBER && S.render[7] > 0.0f) return true;
    return false;
}

// normalAt in straight-line form (shaders/Shaders.metal:3871-3971).
// orbit_iters (optional) gets the orbit iterations of the analytic or tap
// evaluations (the normal phase of FptSdfProfileStats).
template <int KIND> __device__ float3 normal_direct(float3 p, const DeviceScene &S, uint32_t *orbit_iters = nullptr) {
    if (S.sdf_id == FPT_SDF_MANDELBULBER && S.render[7] > 0.0f && !(S.formula != 0 && S.ext_normal == FPT_CUDA_NORMAL_ANALYTIC))
        return mandel_slow_normal<KIND>(p, S);
    float3 g;
    if ((S.formula != 0 && S.ext_normal == FPT_CUDA_NORMAL_ANALYTIC) ||
        (S.formula == 0 && S.sdf_id == FPT_SDF_PROGRAM)) {
        if (analytic_gradient<KIND>(S, p, g, orbit_iters)) {
            if (S.formula != 0) {
                if (finite3(g) && dot(g, g) > 0.0f) return normalize3(g);
                return mk3(0.f, 1.f, 0.f);
            }
            return normalize3(g);
        }
    }
    float e = normal_epsilon(p, S);
    float3 acc = mk3(0.0f);
    int n = tap_count(S), mode = tap_mode(S);
    for (int k = 0; k < n; ++k) {
        const Eval ev = scene_eval<KIND>(S, p + tap_offset(S, k, e), mode);
        if (orbit_iters) *orbit_iters += uint32_t(ev.iters);
        tap_accumulate(S, k, ev.d, acc);
    }
    if (S.normal_mode != 1u && S.sdf_id == FPT_SDF_MANDELBULBER && !(fmaxf(fabsf(acc.x), fmaxf(fabsf(acc.y), fabsf(acc.z))) > 0.0f))
        acc = mandel_orbit_normal<KIND>(p, e, S);
    return normalize_fd(acc);
}

}  // namespace fpt
