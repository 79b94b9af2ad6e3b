// skip.cuh -- surrogate-skip march: learned step proposals, certified by the exact DE.
//
// A ray at p with exact distance d_p = DE(p) asks the network for the
// distance m at the look-ahead point p + lambda d_p dir and proposes the step
// s = d_p + safety * m.  The exact DE at q = p + s dir decides:
//   s <= d_p + DE(q)   the balls of radius d_p around p and DE(q) around q
//                      hold no surface and overlap, so [p, q] is free:
//                      the ray moves to q (one exact evaluation for s)
//   otherwise          one step of the scene's march rule (march_update's
//                      step, applied to the position the way it applies it)
// lambda adapts per ray: 1.5 s / d_p after an accepted step (rays leaving a
// surface look further ahead each step), 2 after a refusal.
// Every step is certified by the exact DE, so the surrogate only changes how
// far a ray gets per evaluation, never what it hits (where the DE is a lower
// bound of the distance; steps it does not replace visit the plain march's
// positions).  When d_p falls below the hand-over margin the exact march
// resumes the ray with its step count and last step.  Camera rays start at
// the plain march's first step; geometry lies inside the model's box, and a
// camera ray that misses or leaves it is a miss without further evaluation.
//
// Two network engines: tcgen05 (default; 128 rows per CTA, accumulators in
// tensor memory, a CTA-synchronous loop) and mma.sync (32 rows per warp, a
// warp-synchronous loop).  Every iteration each lane adds one network row and
// one exact evaluation.
#pragma once

#include "fpt_march.cuh"
#include "mlp.cuh"
#include "mlp_tc.cuh"
#include "wavefront.cuh"

namespace fpt {

struct SkipArgs {
    mlp::Model M;
    float lo[3], hi[3];          // the model's box (all geometry inside)
    float margin;                // hand over to the exact march below this distance
    float safety;                // scale of the predicted distance in a proposal
    uint32_t max_iters;          // skip iterations per ray before hand-over
    uint32_t use_network;        // 0: box clip only (the march kernel applies it; no skip pass)
    uint32_t engine;             // network engine: kNetTcgen05 or kNetMmaSync
    uint32_t *guard;             // primary-ray pass: error word (bit 2: an MMA did not complete), or null
    const uint32_t *cam_step;    // primary-ray pass: the plain march's first step from the camera (float bits), or null
    unsigned long long *stats;   // kSkipStats counters or null
};

enum SkipStat : int { SK_ROWS = 0, SK_FORWARDS = 1, SK_EXACT = 2, SK_ACCEPT = 3, SK_REJECT = 4, SK_ESCAPE = 5, SK_HANDOVER = 6,
                      SK_DIST = 7, kSkipStats = 8 };

constexpr uint32_t kNetTcgen05 = 0, kNetMmaSync = 1;
constexpr int kSkipWarps = 4;
inline size_t skip_smem_bytes() { return ((sizeof(mlp::SmemWeights) + 127) & ~size_t(127)) + kSkipWarps * sizeof(mlp::WarpForward); }

// Forward slab test: [tn, tf] of the ray inside the box, tn >= 0.
__device__ __forceinline__ bool box_span(const SkipArgs &A, float3 p, float3 d, float &tn, float &tf) {
    tn = 0.0f;
    tf = 3.0e38f;
    const float pv[3] = {p.x, p.y, p.z}, dv[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dv[a] != 0.0f) {
            float inv = 1.0f / dv[a];
            float t0 = (A.lo[a] - pv[a]) * inv, t1 = (A.hi[a] - pv[a]) * inv;
            tn = fmaxf(tn, fminf(t0, t1));
            tf = fminf(tf, fmaxf(t0, t1));
        } else if (pv[a] < A.lo[a] || pv[a] > A.hi[a]) {
            return false;
        }
    }
    return tf >= tn;
}

enum SkipPhase : int { SP_IDLE = 0, SP_EXACT = 1, SP_PROPOSE = 2 };

struct SkipLane {
    float3 origin, dir;   // job start and direction
    float3 pos;           // position, advanced step by step like the exact march's (pos + dir * step)
    float t;              // advance along dir from origin (box exit test)
    float t_exit;         // box exit (advance)
    float d;              // exact distance at pos (SP_PROPOSE)
    float lam;            // look-ahead in units of d
    int phase;
    uint32_t iters;
    int steps;            // march steps from the ray's origin (plain steps and accepted skips)
    float last_step;      // length of the last of them
};

// Starts a lane on a ray: clips to the box.  Returns false when the ray
// never meets the box (a miss; t is left at 0).
// t_start >= 0: the ray starts there (before the box too); t_start < 0: at
// the box entry.
// `steps` / `last_step`: plain-march steps already taken to reach origin +
// t_start dir.
__device__ __forceinline__ bool skip_begin(SkipLane &L, const SkipArgs &A, float3 origin, float3 dir, float t_start, int steps,
                                           float last_step) {
    L.origin = origin;
    L.dir = dir;
    L.t = 0.0f;
    L.iters = 0;
    L.d = 0.0f;
    L.lam = 2.0f;
    float tn, tf;
    if (!box_span(A, origin, dir, tn, tf)) { L.phase = SP_IDLE; return false; }
    if (t_start >= 0.0f) tn = t_start;
    if (tn > tf) { L.phase = SP_IDLE; return false; }
    L.t = tn;
    L.pos = tn > 0.0f ? origin + dir * tn : origin;
    L.steps = steps;
    L.last_step = last_step;
    L.t_exit = tf;
    L.phase = SP_EXACT;
    return true;
}

// Start of a primary ray in the primary-ray pass: the plain march's first
// step from the camera when there is one (see first_step_kernel), else the
// box entry.
__device__ __forceinline__ float first_step_or_entry(const SkipArgs &A) {
    const float s1 = A.cam_step ? bitsf(*A.cam_step) : 0.0f;
    return s1 > 0.0f ? s1 : -1.0f;
}

enum SkipOutcome : int { SO_CONTINUE = 0, SO_HANDOVER = 1, SO_ESCAPE = 2 };

// One step of the scene's march rule (march_update) from the lane's position
// with its exact distance L.d, applied to the position the way the exact
// march applies it, so steps the network does not replace visit the plain
// march's positions.
__device__ __forceinline__ void plain_advance(SkipLane &L, const DeviceScene &S) {
    const float step = S.sdf_id == FPT_SDF_MANDELBULBER ? mandel_march_step(L.d, mandel_threshold(L.pos, S), S) : fabsf(L.d) * 0.99f;
    L.pos = L.pos + L.dir * step;
    L.t += step;
    ++L.steps;
    L.last_step = step;
}

// The network query of a lane in SP_PROPOSE: the look-ahead point p + lam d
// dir, normalised to the model box (other lanes query their position; the
// row is computed but not used).  Returns whether the lane proposes.
__device__ __forceinline__ bool skip_query(const SkipLane &L, const SkipArgs &A, float u[3]) {
    const bool propose = A.use_network && L.phase == SP_PROPOSE;
    const float3 p = L.pos;
    const float3 q0 = propose ? p + L.dir * (L.lam * L.d) : p;
    u[0] = (q0.x - A.M.center[0]) * A.M.inv_half[0];
    u[1] = (q0.y - A.M.center[1]) * A.M.inv_half[1];
    u[2] = (q0.z - A.M.center[2]) * A.M.inv_half[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) u[k] = fminf(fmaxf(u[k], -4.0f), 4.0f);
    return propose;
}

// The rest of an iteration once the network distance m (world units) of a
// proposing lane is known: the proposal, its certification by one exact
// evaluation, and the hand-over / escape decision.
template <int KIND>
__device__ __forceinline__ int skip_advance(SkipLane &L, const DeviceScene &S, const SkipArgs &A, bool propose, float m,
                                            uint32_t &c_exact, uint32_t &c_acc, uint32_t &c_rej) {
    if (L.phase == SP_IDLE) return SO_CONTINUE;
    bool cand = false;
    float s = 0.0f;
    if (propose) {
        s = L.d + A.safety * fmaxf(m, 0.0f);
        if (s > 1.25f * L.d && isfinite(s)) {
            cand = true;
        } else {   // no useful proposal: the plain step
            plain_advance(L, S);
            L.phase = SP_EXACT;
        }
    } else if (L.phase == SP_PROPOSE) {   // box-only mode: plain steps
        plain_advance(L, S);
    }
    const float3 q = L.pos + L.dir * s;
    const float de = scene_eval<KIND>(S, cand ? q : L.pos, EV_MAP).d;
    ++c_exact;
    if (cand) {
        if (s <= L.d + de && isfinite(de)) {
            L.lam = fminf(fmaxf(1.5f * s / L.d, 2.0f), 32.0f);
            L.pos = q;
            L.t += s;
            ++L.steps;
            L.last_step = s;
            L.d = de;
            ++c_acc;
        } else {
            L.lam = 2.0f;
            plain_advance(L, S);
            L.phase = SP_EXACT;
            ++c_rej;
        }
    } else {
        L.d = de;
        L.phase = SP_PROPOSE;
    }
    if (L.t >= L.t_exit) return SO_ESCAPE;
    // Hand over near a surface.  (Keeping rays that leave a surface in the
    // skip pass until their distance stops growing cost more exact
    // evaluations than it saved on the power-8 Mandelbulb at 1080p.)
    if (L.phase == SP_PROPOSE && (!isfinite(L.d) || fabsf(L.d) < A.margin)) return SO_HANDOVER;
    if (++L.iters >= A.max_iters) return SO_HANDOVER;
    return SO_CONTINUE;
}

// One warp-synchronous iteration for all 32 lanes (every lane must call it;
// lanes with phase SP_IDLE only lend their network row).
template <int KIND>
__device__ __forceinline__ int skip_step(SkipLane &L, const DeviceScene &S, const SkipArgs &A, const mlp::SmemWeights &sw,
                                         mlp::WarpForward &wf, int lane, uint32_t &c_rows, uint32_t &c_fwd, uint32_t &c_exact,
                                         uint32_t &c_acc, uint32_t &c_rej) {
    float u[3];
    const bool propose = skip_query(L, A, u);
    float m = 0.0f;
    if (__any_sync(0xffffffffu, propose)) {
        m = mlp::forward32(sw, wf, u, lane) * A.M.label_scale;
        if (lane == 0) ++c_fwd;
        if (propose) ++c_rows;
    }
    return skip_advance<KIND>(L, S, A, propose, m, c_exact, c_acc, c_rej);
}

__device__ __forceinline__ void skip_flush_stats(const SkipArgs &A, int lane, uint32_t rows, uint32_t fwd, uint32_t exact,
                                                 uint32_t acc, uint32_t rej, uint32_t esc, uint32_t hand) {
    if (!A.stats) return;
    uint32_t v[7] = {rows, fwd, exact, acc, rej, esc, hand};
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        uint32_t s = v[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s) atomicAdd(A.stats + k, (unsigned long long)s);
    }
}

// Takes jobs for the warp's idle lanes from the skip queue (camera rays that
// enter the box, queued by the camera kernel): warp-synchronous, one atomic
// per warp.
__device__ __forceinline__ void skip_refill(SkipLane &L, const SkipArgs &A, const WaveParams &W, uint32_t total, int lane,
                                            bool &retired, uint32_t &job, uint32_t &c_esc) {
    const unsigned FULL = 0xffffffffu;
    const bool need = L.phase == SP_IDLE && !retired;
    const unsigned ballot = __ballot_sync(FULL, need);
    if (!ballot) return;
    const uint32_t leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == int(leader)) base = atomicAdd(&W.counters[C_SKIP], (unsigned)__popc(ballot));
    base = __shfl_sync(FULL, base, leader);
    if (!need) return;
    const uint32_t idx = base + __popc(ballot & ((1u << lane) - 1u));
    if (idx >= total) {
        retired = true;
        return;
    }
    const float4 o = W.q_skip[idx].origin, d = W.q_skip[idx].dir;
    job = fbits(o.w);
    if (!skip_begin(L, A, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), 0.0f, int(d.w), 0.0f)) {   // only where the camera kernel's start lies on the box exit
        ++c_esc;
        W.paths[job].color.w = bitsf(fbits(W.paths[job].color.w) | PF_ESCAPED);
    }
}

// Writes the outcome of a lane whose skip ended (escape or hand-over) into
// its path record and idles the lane.
__device__ __forceinline__ void skip_finish(SkipLane &L, const WaveParams &W, int out, uint32_t job, uint32_t &c_esc, uint32_t &c_hand) {
    if (out == SO_ESCAPE) ++c_esc; else ++c_hand;
    const bool known = out == SO_HANDOVER && L.phase == SP_PROPOSE;   // L.d is the exact distance here
    PathRec &R = W.paths[job];
    const float3 p = L.pos;
    R.pos = make_float4(p.x, p.y, p.z, R.pos.w);
    R.shadow.w = float(L.steps);
    uint32_t st = fbits(R.color.w);
    if (out == SO_ESCAPE) st |= PF_ESCAPED;
    if (known) {
        R.grad.w = L.d;
        st |= PF_KNOWN_D;
    }
    R.color.w = bitsf(st);
    L.phase = SP_IDLE;
}

// Wavefront pass before the first march pass: advances the camera rays of
// the skip queue before the exact march kernel takes them.  A ray's R.pos
// moves; an escape sets PF_ESCAPED (the march kernel then classifies the ray
// as a miss without evaluating); a hand-over with the exact distance in hand
// sets PF_KNOWN_D.  Jobs are taken with per-lane regeneration from counter
// C_SKIP.  Network on mma.sync, one warp (32 rows) at a time.
template <int KIND>
__global__ void __launch_bounds__(32 * kSkipWarps, 3) skip_march_kernel(WaveParams W, SkipArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mlp::SmemWeights &sw = *reinterpret_cast<mlp::SmemWeights *>(smem_raw);
    mlp::WarpForward *wf_all =
        reinterpret_cast<mlp::WarpForward *>(smem_raw + ((sizeof(mlp::SmemWeights) + 127) & ~size_t(127)));
    const DeviceScene &S = c_scene;
    const uint32_t total = W.counters[C_SKIPN];
    if (total == 0u) return;
    mlp::load_weights(sw, A.M);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    mlp::WarpForward &wf = wf_all[warp];
    const unsigned FULL = 0xffffffffu;
    SkipLane L;
    L.phase = SP_IDLE;
    bool retired = false;
    uint32_t job = 0;
    uint32_t c_rows = 0, c_fwd = 0, c_exact = 0, c_acc = 0, c_rej = 0, c_esc = 0, c_hand = 0;
    uint32_t trips = 0;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (loop_guard(trips, t0, W.counters, W.loop_limit_ns)) break;
        skip_refill(L, A, W, total, lane, retired, job, c_esc);
        if (!__any_sync(FULL, L.phase != SP_IDLE)) {
            if (__all_sync(FULL, retired)) break;
            continue;
        }
        const int out = skip_step<KIND>(L, S, A, sw, wf, lane, c_rows, c_fwd, c_exact, c_acc, c_rej);
        if (L.phase != SP_IDLE && out != SO_CONTINUE) skip_finish(L, W, out, job, c_esc, c_hand);
    }
    skip_flush_stats(A, lane, c_rows, c_fwd, c_exact, c_acc, c_rej, c_esc, c_hand);
}

// Job feed of the CTA-synchronous pass.  A stall of one warp stalls the
// whole CTA there, so refills must not wait on memory: each warp takes job
// indices from a chunk it claimed one chunk ahead (the claim's atomic result
// is read only when the current chunk runs out), and each lane loads its next
// job one job ahead (the loads are consumed when the lane's current ray ends).
constexpr uint32_t kSkipChunk = 64;
struct SkipFeed {
    uint32_t cur_base, taken, next_base;   // the same in every lane of the warp
    uint32_t pending;                      // lane 0: claim of the chunk after next (read at the next roll-over)
};
__device__ __forceinline__ void feed_init(SkipFeed &F, const WaveParams &W, int lane) {
    uint32_t a = 0;
    if (lane == 0) a = atomicAdd(&W.counters[C_SKIP], 2u * kSkipChunk);
    a = __shfl_sync(0xffffffffu, a, 0);
    F.cur_base = a;
    F.next_base = a + kSkipChunk;
    F.taken = 0;
    F.pending = 0;
    if (lane == 0) F.pending = atomicAdd(&W.counters[C_SKIP], kSkipChunk);
}
// The next job index of every lane with `need` (warp-synchronous).
__device__ __forceinline__ uint32_t feed_take(SkipFeed &F, bool need, const WaveParams &W, int lane) {
    const unsigned ballot = __ballot_sync(0xffffffffu, need);
    const uint32_t pos = F.taken + __popc(ballot & ((1u << lane) - 1u));
    const uint32_t idx = pos < kSkipChunk ? F.cur_base + pos : F.next_base + (pos - kSkipChunk);
    F.taken += __popc(ballot);
    if (F.taken >= kSkipChunk) {   // at most 32 indices spill into the next chunk
        F.taken -= kSkipChunk;
        F.cur_base = F.next_base;
        F.next_base = __shfl_sync(0xffffffffu, F.pending, 0);
        if (lane == 0) F.pending = atomicAdd(&W.counters[C_SKIP], kSkipChunk);
    }
    return idx;
}

// The same pass with the network on the 5th-generation tensor cores: the
// loop is CTA-synchronous, and each iteration in which any lane of the
// 128-thread CTA proposes runs one 128-row forward pass (mlp::tc_forward).
// Guard word bits: 1 = loop time limit, 2 = an MMA did not complete.
template <int KIND>
__global__ void __launch_bounds__(mlp::kTcRows, 4) skip_march_tc_kernel(WaveParams W, SkipArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mlp::TcSmem &sm = *reinterpret_cast<mlp::TcSmem *>(smem_raw);
    const DeviceScene &S = c_scene;
    const uint32_t total = W.counters[C_SKIPN];
    if (total == 0u) return;
    mlp::tc_setup(sm, A.M);
    const int lane = threadIdx.x & 31;
    SkipLane L;
    L.phase = SP_IDLE;
    bool fed_out = false, has_next = false, fail = false;
    float4 next_o = make_float4(0.f, 0.f, 0.f, 0.f), next_d = next_o;
    uint32_t job = 0, phase = 0;
    uint32_t c_rows = 0, c_fwd = 0, c_exact = 0, c_acc = 0, c_rej = 0, c_esc = 0, c_hand = 0;
    SkipFeed F;
    feed_init(F, W, lane);
    uint32_t trips = 0;
    const unsigned long long t0 = global_ns();
    while (true) {
        if ((++trips & 1023u) == 0u) {   // the same trip in every thread
            if (__syncthreads_or(global_ns() - t0 > W.loop_limit_ns)) {
                if (threadIdx.x == 0) atomicOr(W.counters + C_GUARD, 1u);
                break;
            }
        }
        // An idle lane starts the job it loaded earlier, then loads its next one.
        if (L.phase == SP_IDLE && has_next) {
            has_next = false;
            job = fbits(next_o.w);
            if (!skip_begin(L, A, mk3(next_o.x, next_o.y, next_o.z), mk3(next_d.x, next_d.y, next_d.z), 0.0f, int(next_d.w), 0.0f)) {
                ++c_esc;   // only where the camera kernel's start lies on the box exit
                W.paths[job].color.w = bitsf(fbits(W.paths[job].color.w) | PF_ESCAPED);
            }
        }
        {
            const bool want = !has_next && !fed_out;
            const uint32_t idx = feed_take(F, want, W, lane);
            if (want) {
                if (idx < total) {
                    next_o = W.q_skip[idx].origin;
                    next_d = W.q_skip[idx].dir;
                    has_next = true;
                } else {
                    fed_out = true;
                }
            }
        }
        const bool retired = L.phase == SP_IDLE && !has_next && fed_out;
        if (!__syncthreads_or(L.phase != SP_IDLE)) {
            if (__syncthreads_and(retired)) break;
            continue;
        }
        float u[3];
        const bool propose = skip_query(L, A, u);
        float m = 0.0f;
        if (__syncthreads_or(propose)) {
            m = mlp::tc_forward(sm, phase, u, fail) * A.M.label_scale;
            if (fail) break;   // the same in every thread
            if (lane == 0) ++c_fwd;
            if (propose) ++c_rows;
        }
        const int out = skip_advance<KIND>(L, S, A, propose, m, c_exact, c_acc, c_rej);
        if (L.phase != SP_IDLE && out != SO_CONTINUE) skip_finish(L, W, out, job, c_esc, c_hand);
    }
    mlp::tc_teardown(sm);
    if (fail && threadIdx.x == 0) atomicOr(W.counters + C_GUARD, 2u);
    skip_flush_stats(A, lane, c_rows, c_fwd, c_exact, c_acc, c_rej, c_esc, c_hand);
}

// Primary rays with the surrogate skip in front of the exact march (the
// counterpart of trace_primary_kernel): per pixel distance, normal, exact
// evaluations (skip + march) and hit flag.
template <int KIND>
__global__ void __launch_bounds__(32 * kSkipWarps, 3) skip_primary_kernel(const DeviceScene *scene, SkipArgs A,
                                                                          FptCudaPrimaryHit *hits) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mlp::SmemWeights &sw = *reinterpret_cast<mlp::SmemWeights *>(smem_raw);
    mlp::WarpForward *wf_all =
        reinterpret_cast<mlp::WarpForward *>(smem_raw + ((sizeof(mlp::SmemWeights) + 127) & ~size_t(127)));
    const DeviceScene &S = *scene;
    mlp::load_weights(sw, A.M);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    mlp::WarpForward &wf = wf_all[warp];
    const uint32_t pixels = S.width * S.height;
    uint32_t c_rows = 0, c_fwd = 0, c_exact = 0, c_acc = 0, c_rej = 0, c_esc = 0, c_hand = 0;
    for (uint32_t base = (blockIdx.x * kSkipWarps + warp) * 32u; base < pixels; base += gridDim.x * kSkipWarps * 32u) {
        const uint32_t i = base + lane;
        const bool valid = i < pixels;
        const uint32_t gx = valid ? i % S.width : 0u, gy = valid ? i / S.width : 0u;
        float2 uv = screen_uv(gx, gy, S);
        PathRng rng;
        rng.init(false, 0u, 0u, 0u, uv.x, uv.y);
        float3 rp = mk3(0.f), dr = mk3(0.f, 0.f, 1.f);
        bool ray = valid && camera_ray(S, uv, rng, false, rp, dr);
        SkipLane L;
        L.phase = SP_IDLE;
        bool escaped = false;
        uint32_t exact0 = c_exact;
        const float t_start = first_step_or_entry(A);
        if (ray && !skip_begin(L, A, rp, dr, t_start, t_start > 0.0f ? 1 : 0, fmaxf(t_start, 0.0f))) escaped = true;
        while (__any_sync(0xffffffffu, L.phase != SP_IDLE)) {
            int out = skip_step<KIND>(L, S, A, sw, wf, lane, c_rows, c_fwd, c_exact, c_acc, c_rej);
            if (L.phase != SP_IDLE && out != SO_CONTINUE) {
                if (out == SO_ESCAPE) { escaped = true; ++c_esc; } else ++c_hand;
                L.phase = SP_IDLE;
            }
        }
        if (!valid) continue;
        FptCudaPrimaryHit h;
        h.distance = 0.0f; h.normal[0] = h.normal[1] = h.normal[2] = 0.0f; h.steps = 0; h.hit = 0;
        if (ray) {
            if (escaped) {
                h.distance = S.render[4];
                h.steps = c_exact - exact0;
            } else {
                March m = march_loop_from<KIND>(S, rp, L.pos, dr, int(S.render[1]), S.render[3], 0.0002f, L.steps, L.last_step);
                float travel = len3(m.pos - rp);
                bool hit = m.found && isfinite(travel) && travel < S.render[4] * 0.99f;
                h.distance = travel;
                h.steps = uint32_t(m.steps) + (c_exact - exact0);
                h.hit = hit ? 1u : 0u;
                if (hit) {
                    float3 n = normal_direct<KIND>(m.pos, S);
                    h.normal[0] = n.x; h.normal[1] = n.y; h.normal[2] = n.z;
                }
            }
        }
        hits[i] = h;
    }
    skip_flush_stats(A, lane, c_rows, c_fwd, c_exact, c_acc, c_rej, c_esc, c_hand);
}

// skip_primary_kernel with the network on tcgen05: 128 pixels per CTA
// iteration, CTA-synchronous skip loop.
template <int KIND>
__global__ void __launch_bounds__(mlp::kTcRows, 4) skip_primary_tc_kernel(const DeviceScene *scene, SkipArgs A,
                                                                          FptCudaPrimaryHit *hits) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mlp::TcSmem &sm = *reinterpret_cast<mlp::TcSmem *>(smem_raw);
    const DeviceScene &S = *scene;
    mlp::tc_setup(sm, A.M);
    const int lane = threadIdx.x & 31;
    const uint32_t pixels = S.width * S.height;
    uint32_t phase = 0;
    bool fail = false;
    uint32_t c_rows = 0, c_fwd = 0, c_exact = 0, c_acc = 0, c_rej = 0, c_esc = 0, c_hand = 0;
    for (uint32_t base = blockIdx.x * uint32_t(mlp::kTcRows); base < pixels; base += gridDim.x * uint32_t(mlp::kTcRows)) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < pixels;
        const uint32_t gx = valid ? i % S.width : 0u, gy = valid ? i / S.width : 0u;
        float2 uv = screen_uv(gx, gy, S);
        PathRng rng;
        rng.init(false, 0u, 0u, 0u, uv.x, uv.y);
        float3 rp = mk3(0.f), dr = mk3(0.f, 0.f, 1.f);
        bool ray = valid && camera_ray(S, uv, rng, false, rp, dr);
        SkipLane L;
        L.phase = SP_IDLE;
        bool escaped = false;
        uint32_t exact0 = c_exact;
        const float t_start = first_step_or_entry(A);
        if (ray && !skip_begin(L, A, rp, dr, t_start, t_start > 0.0f ? 1 : 0, fmaxf(t_start, 0.0f))) escaped = true;
        while (__syncthreads_or(L.phase != SP_IDLE)) {
            float u[3];
            const bool propose = skip_query(L, A, u);
            float m = 0.0f;
            if (__syncthreads_or(propose)) {
                m = mlp::tc_forward(sm, phase, u, fail) * A.M.label_scale;
                if (fail) break;   // the same in every thread
                if (lane == 0) ++c_fwd;
                if (propose) ++c_rows;
            }
            const int out = skip_advance<KIND>(L, S, A, propose, m, c_exact, c_acc, c_rej);
            if (L.phase != SP_IDLE && out != SO_CONTINUE) {
                if (out == SO_ESCAPE) { escaped = true; ++c_esc; } else ++c_hand;
                L.phase = SP_IDLE;
            }
        }
        if (fail) break;
        if (!valid) continue;
        FptCudaPrimaryHit h;
        h.distance = 0.0f; h.normal[0] = h.normal[1] = h.normal[2] = 0.0f; h.steps = 0; h.hit = 0;
        if (ray) {
            if (escaped) {
                h.distance = S.render[4];
                h.steps = c_exact - exact0;
            } else {
                March m = march_loop_from<KIND>(S, rp, L.pos, dr, int(S.render[1]), S.render[3], 0.0002f, L.steps, L.last_step);
                float travel = len3(m.pos - rp);
                bool hit = m.found && isfinite(travel) && travel < S.render[4] * 0.99f;
                h.distance = travel;
                h.steps = uint32_t(m.steps) + (c_exact - exact0);
                h.hit = hit ? 1u : 0u;
                if (hit) {
                    float3 n = normal_direct<KIND>(m.pos, S);
                    h.normal[0] = n.x; h.normal[1] = n.y; h.normal[2] = n.z;
                }
            }
        }
        hits[i] = h;
    }
    mlp::tc_teardown(sm);
    if (fail && threadIdx.x == 0 && A.guard) atomicOr(A.guard, 2u);
    skip_flush_stats(A, lane, c_rows, c_fwd, c_exact, c_acc, c_rej, c_esc, c_hand);
}

}  // namespace fpt
