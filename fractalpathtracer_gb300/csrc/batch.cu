// batch.cu -- many scenes in one render: persistent passes over all scenes,
// one CUDA graph per spp pass, and the launch-shape autotuner.
//
// A batch holds scenes of uneven resolution and iteration count (extension
// formulas: Mandelbulb of any power, Mandelbox, Menger fold, hybrids).  Every
// pass renders sample p of every scene: the camera kernel maps a work index
// to (scene, pixel) through a prefix table, the persistent march kernel
// takes path and shadow rays of all scenes from one queue (a path carries its
// scene index in its state word), and the pass ends with the in-order
// running-mean update of every pixel.  The launches of one pass (per wave:
// counter reset, camera, bounces + 1 march passes, bounces shade passes,
// finalize; then reduce and the pass-index increment) are captured once into
// a CUDA graph and replayed spp times; the pass index lives in device memory,
// so the same graph serves every sample.
//
// Autotuner: the march kernel is instantiated with several launch shapes
// (block size x register cap through __launch_bounds__); together with the
// wavefront length (paths per wave) and the march's finish/refill group size
// they form the candidates.  Candidates are
// timed on the batch itself in interleaved rounds (median per candidate); a
// candidate replaces the default only when it is faster by a margin, and the
// choice is kept for the batch's workload key (the measured-selection
// discipline of the reference's backend selector, src/main.rs:37-47,
// 983-1305).
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "bridge_internal.h"
#include "render_impl.cuh"

namespace fpt {
namespace {

using MarchFn = void (*)(WaveParams, int);

struct MarchVariant {
    int block, minb;
    MarchFn fn;
};

const MarchVariant kVariants[] = {
    {128, 7, march_kernel<KIND_EXT, true, 128, 7>},   // default: <= 72 registers
    {128, 8, march_kernel<KIND_EXT, true, 128, 8>},   // <= 64 registers
    {128, 5, march_kernel<KIND_EXT, true, 128, 5>},   // <= 102 registers
    {256, 3, march_kernel<KIND_EXT, true, 256, 3>},   // <= 85 registers, 256-thread blocks
};
constexpr int kVariantCount = int(sizeof(kVariants) / sizeof(kVariants[0]));
constexpr double kTuneMargin = 0.03;   // a candidate must beat the default by 3%

struct TuneChoice {
    int variant = 0;
    uint32_t wave_paths = 0;   // 0: all paths of a pass in one wave (capped at 16M)
    uint32_t refill = 0;       // finish/refill group of the march (0: the kernel's default)
};

std::map<uint64_t, TuneChoice> &tuned() {
    static std::map<uint64_t, TuneChoice> m;
    return m;
}

struct BatchState {
    DeviceScene *scenes = nullptr; size_t cap_scenes = 0;
    uint32_t *tables = nullptr; size_t cap_tables = 0;   // work_base | pixel_base | pass
    float4 *accum = nullptr; size_t cap_accum = 0;
    float4 *sample_rgb = nullptr; size_t cap_sample = 0;
    uchar4 *rgba = nullptr; size_t cap_rgba = 0;
};
BatchState &bstate() {
    static BatchState b;
    return b;
}

struct BatchPlan {
    std::vector<DeviceScene> scenes;
    std::vector<uint32_t> work_base, pixel_base;
    uint32_t spp = 0, max_bounces = 0;
    uint64_t pixels = 0, work = 0, key = 0;
};

uint64_t fnv(uint64_t h, uint64_t v) {
    for (int i = 0; i < 8; ++i) {
        h ^= (v >> (8 * i)) & 0xffu;
        h *= 1099511628211ull;
    }
    return h;
}

bool make_plan(const FptRenderConfig *configs, const FptCudaSceneExt *exts, size_t count, BatchPlan &P, char *error,
               size_t error_len) {
    if (!configs || !exts || count == 0) { set_error(error, error_len, "a batch needs configs, extensions and count > 0"); return false; }
    if (count > 65535) { set_error(error, error_len, "a batch holds at most 65535 scenes"); return false; }
    P.scenes.resize(count);
    P.work_base.assign(count + 1, 0);
    P.pixel_base.assign(count + 1, 0);
    uint64_t key = 1469598103934665603ull;
    for (size_t k = 0; k < count; ++k) {
        const FptRenderConfig &c = configs[k];
        const FptCudaSceneExt &e = exts[k];
        if (c.width == 0 || c.height == 0) { set_error(error, error_len, "scene %zu: invalid size", k); return false; }
        if (e.formula == 0) { set_error(error, error_len, "scene %zu: batched scenes take extension formulas", k); return false; }
        if (e.sky_width > 0) { set_error(error, error_len, "scene %zu: batched scenes take no sky image", k); return false; }
        if (e.surrogate) { set_error(error, error_len, "scene %zu: batched scenes do not run the surrogate skip", k); return false; }
        if (c.renderer_backend != FPT_RENDERER_SDF) { set_error(error, error_len, "scene %zu: batched scenes use the SDF renderer", k); return false; }
        FptRenderConfig h = c;
        if (!hydrate_hdri(h, error, error_len)) return false;
        if (!compile_scene(h, &e, P.scenes[k], error, error_len)) return false;
        const DeviceScene &S = P.scenes[k];
        if (k == 0) P.spp = S.samples;
        if (S.samples != P.spp || S.samples == 0) {
            set_error(error, error_len, "scene %zu: every scene of a batch takes the same sample count (> 0)", k);
            return false;
        }
        P.max_bounces = std::max(P.max_bounces, S.bounces);
        const uint64_t tiles = uint64_t((S.width + 7u) / 8u) * ((S.height + 3u) / 4u);
        const uint64_t work = P.work_base[k] + tiles * 32u, pix = P.pixel_base[k] + uint64_t(S.width) * S.height;
        if (work > 0xffffffffull || pix > 0xffffffffull) { set_error(error, error_len, "batch too large"); return false; }
        P.work_base[k + 1] = uint32_t(work);
        P.pixel_base[k + 1] = uint32_t(pix);
        key = fnv(key, S.width);
        key = fnv(key, S.height);
        key = fnv(key, S.kind);
        key = fnv(key, S.iterations);
        key = fnv(key, S.bounces);
    }
    P.work = P.work_base[count];
    P.pixels = P.pixel_base[count];
    P.key = fnv(fnv(key, P.spp), count);
    return true;
}

// Uploads the scenes and tables and sizes the buffers.
bool upload_plan(const BatchPlan &P, uint32_t wave_paths, char *error, size_t error_len) {
    Context &c = ctx();
    BatchState &B = bstate();
    const size_t n = P.scenes.size();
    if (!ensure_buffer((void **)&B.scenes, &B.cap_scenes, n * sizeof(DeviceScene), error, error_len) ||
        !ensure_buffer((void **)&B.tables, &B.cap_tables, (2 * (n + 1) + 1) * sizeof(uint32_t), error, error_len) ||
        !ensure_buffer((void **)&B.accum, &B.cap_accum, P.pixels * sizeof(float4), error, error_len) ||
        !ensure_buffer((void **)&B.sample_rgb, &B.cap_sample, P.pixels * sizeof(float4), error, error_len) ||
        !ensure_buffer(&c.wave, &c.cap_wave, wave_scratch_bytes(wave_paths), error, error_len) ||
        !ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len))
        return false;
    std::vector<uint32_t> tables(2 * (n + 1) + 1, 0u);
    std::copy(P.work_base.begin(), P.work_base.end(), tables.begin());
    std::copy(P.pixel_base.begin(), P.pixel_base.end(), tables.begin() + (n + 1));
    return check(cudaMemcpyAsync(B.scenes, P.scenes.data(), n * sizeof(DeviceScene), cudaMemcpyHostToDevice, c.stream), "scene upload",
                 error, error_len) &&
           check(cudaMemcpyAsync(B.tables, tables.data(), tables.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream),
                 "table upload", error, error_len);
}

uint32_t wave_for(const BatchPlan &P, uint32_t requested) {
    uint64_t cap = requested ? requested : (uint64_t(16) << 20);
    return uint32_t(std::max<uint64_t>(std::min<uint64_t>(cap, P.work), 32));
}

// Launches one pass of the batch on `st` (captured into the graph).  Returns
// the number of kernel launches.
uint32_t launch_pass(const BatchPlan &P, const MarchVariant &V, uint32_t wave_paths, uint32_t refill, cudaStream_t st) {
    Context &c = ctx();
    BatchState &B = bstate();
    const size_t n = P.scenes.size();
    WaveParams W{};
    W.scene = B.scenes;
    W.scenes = B.scenes;
    W.n_scenes = uint32_t(n);
    W.work_base = B.tables;
    W.pixel_base = B.tables + (n + 1);
    W.pass = B.tables + 2 * (n + 1);
    W.sample_count = 1;
    W.sample_rgb = B.sample_rgb;
    W.counters = c.counter;
    W.profile = nullptr;
    W.box_on = 0;
    W.refill_batch = refill;
    const uint32_t cap = wave_paths;
    char *base = static_cast<char *>(c.wave);
    W.paths = reinterpret_cast<PathRec *>(base);
    W.q_shadow[0] = reinterpret_cast<ShadowJob *>(base + size_t(cap) * 96);
    W.q_shadow[1] = W.q_shadow[0] + cap;
    W.q_march[0] = reinterpret_cast<uint32_t *>(base + size_t(cap) * (96 + 128));
    W.q_march[1] = W.q_march[0] + cap;
    W.q_shade = W.q_march[1] + cap;
    W.q_skip = nullptr;
    W.loop_limit_ns = kLoopLimitNs;
    W.skip_queue = 0u;
    int sms = 0, dev = 0, per_sm = 0, shade_per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, V.fn, V.block, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade_per_sm, shade_kernel<KIND_EXT, true>, 128, 0);
    const int march_blocks = sms * std::max(per_sm, 1);
    const int shade_blocks = sms * std::max(shade_per_sm, 1);
    uint32_t launches = 0;
    for (uint64_t wb = 0; wb < P.work; wb += cap) {
        W.wave_base = uint32_t(wb);
        W.n_paths = uint32_t(std::min<uint64_t>(cap, P.work - wb));
        cudaMemsetAsync(W.counters, 0, C_COUNT * sizeof(uint32_t), st);
        camera_kernel<true><<<std::min<uint32_t>((W.n_paths + 255u) / 256u, uint32_t(sms) * 16u), 256, 0, st>>>(W);
        ++launches;
        for (uint32_t b = 0; b <= P.max_bounces; ++b) {
            const int cur = int(b & 1u);
            reset_counters_kernel<<<1, 32, 0, st>>>(W.counters, cur ^ 1);
            V.fn<<<march_blocks, V.block, 0, st>>>(W, cur);
            launches += 2;
            if (b < P.max_bounces) {
                shade_kernel<KIND_EXT, true><<<shade_blocks, 128, 0, st>>>(W, cur);
                ++launches;
            }
        }
        finalize_kernel<true><<<(W.n_paths + 255u) / 256u, 256, 0, st>>>(W);
        ++launches;
    }
    reduce_pass_kernel<<<uint32_t((P.pixels + 255) / 256), 256, 0, st>>>(B.sample_rgb, B.accum, uint32_t(P.pixels), W.pass);
    advance_pass_kernel<<<1, 32, 0, st>>>(B.tables + 2 * (n + 1));
    return launches + 2;
}

// Captures one pass into a graph.
bool capture_pass(const BatchPlan &P, const MarchVariant &V, uint32_t wave_paths, uint32_t refill, cudaGraphExec_t &exec,
                  uint32_t &launches,
                  char *error, size_t error_len) {
    Context &c = ctx();
    cudaGraph_t graph = nullptr;
    if (!check(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal), "graph capture", error, error_len)) return false;
    launches = launch_pass(P, V, wave_paths, refill, c.stream);
    cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
    if (!check(e, "graph capture", error, error_len)) return false;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    return check(e, "graph instantiation", error, error_len);
}

// Renders all spp passes with one graph; returns the device time of the replays.
bool render_plan(const BatchPlan &P, const TuneChoice &choice, float &ms, uint32_t &launches_per_pass, double &build_ms,
                 char *error, size_t error_len) {
    Context &c = ctx();
    BatchState &B = bstate();
    const int variant = choice.variant;
    const uint32_t wave = wave_for(P, choice.wave_paths);
    if (!upload_plan(P, wave, error, error_len)) return false;
    const size_t n = P.scenes.size();
    // focus prepass of scenes without a focus distance (outside the graph)
    for (size_t k = 0; k < n; ++k)
        if (P.scenes[k].focus_distance <= 0.0f) focus_kernel<KIND_EXT><<<1, 32, 0, c.stream>>>(B.scenes + k);
    if (!check(cudaMemsetAsync(B.tables + 2 * (n + 1), 0, sizeof(uint32_t), c.stream), "pass reset", error, error_len) ||
        !check(cudaMemsetAsync(c.counter, 0, 64, c.stream), "counter reset", error, error_len))
        return false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c.stream);
    cudaGraphExec_t exec = nullptr;
    const bool ok = capture_pass(P, kVariants[variant], wave, choice.refill, exec, launches_per_pass, error, error_len);
    cudaEventRecord(e1, c.stream);
    float bms = 0.0f;
    if (ok) {
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&bms, e0, e1);
    }
    build_ms = bms;
    bool good = ok;
    if (ok) {
        cudaEventRecord(e0, c.stream);
        for (uint32_t s = 0; s < P.spp && good; ++s) good = check(cudaGraphLaunch(exec, c.stream), "graph launch", error, error_len);
        cudaEventRecord(e1, c.stream);
        good = good && check(cudaStreamSynchronize(c.stream), "batch render", error, error_len);
        if (good) cudaEventElapsedTime(&ms, e0, e1);
        uint32_t guard = 0;
        if (good && check(cudaMemcpy(&guard, c.counter + C_GUARD, sizeof(guard), cudaMemcpyDeviceToHost), "guard readback", error,
                          error_len) && guard) {
            set_error(error, error_len, "a persistent march loop exceeded its 10 s limit and stopped (batch render aborted)");
            good = false;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return good;
}

}  // namespace
}  // namespace fpt

using namespace fpt;

extern "C" {

int fpt_cuda_render_batch(const struct FptRenderConfig *configs, const struct FptCudaSceneExt *exts, size_t count,
                          float *linear_output, size_t linear_len, uint8_t *rgba_output, size_t rgba_len,
                          struct FptCudaBatchStats *stats, char *error, size_t error_len) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    BatchPlan P;
    if (!make_plan(configs, exts, count, P, error, error_len)) return 1;
    if (linear_output && linear_len < P.pixels * 4) { set_error(error, error_len, "linear output too small (need %llu floats)", (unsigned long long)(P.pixels * 4)); return 1; }
    if (rgba_output && rgba_len < P.pixels * 4) { set_error(error, error_len, "rgba output too small (need %llu bytes)", (unsigned long long)(P.pixels * 4)); return 1; }
    TuneChoice choice;
    bool was_tuned = false;
    auto it = tuned().find(P.key);
    if (it != tuned().end()) { choice = it->second; was_tuned = true; }
    float ms = 0.0f;
    uint32_t launches = 0;
    double build_ms = 0.0;
    if (!render_plan(P, choice, ms, launches, build_ms, error, error_len)) return 1;
    Context &c = ctx();
    BatchState &B = bstate();
    if (linear_output &&
        !check(cudaMemcpy(linear_output, B.accum, P.pixels * sizeof(float4), cudaMemcpyDeviceToHost), "linear readback", error, error_len))
        return 1;
    if (rgba_output) {
        if (!ensure_buffer((void **)&B.rgba, &B.cap_rgba, P.pixels * sizeof(uchar4), error, error_len)) return 1;
        for (size_t k = 0; k < count; ++k)
            launch_present(B.scenes + k, P.scenes[k].width, P.scenes[k].height, B.accum + P.pixel_base[k], B.rgba + P.pixel_base[k],
                           c.stream);
        if (!check(cudaStreamSynchronize(c.stream), "present", error, error_len) ||
            !check(cudaMemcpy(rgba_output, B.rgba, P.pixels * 4, cudaMemcpyDeviceToHost), "image readback", error, error_len))
            return 1;
    }
    if (stats) {
        const MarchVariant &V = kVariants[choice.variant];
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, V.fn);
        stats->elapsed_ms = ms;
        stats->build_ms = build_ms;
        stats->paths = uint64_t(P.pixels) * P.spp;
        stats->scenes = uint32_t(count);
        stats->passes = P.spp;
        stats->graph_launches = P.spp;
        stats->kernel_launches_per_pass = launches;
        stats->block_size = uint32_t(V.block);
        stats->registers = uint32_t(fa.numRegs);
        stats->wave_paths = wave_for(P, choice.wave_paths);
        stats->refill = choice.refill;
        stats->tuned = was_tuned ? 1u : 0u;
        stats->workload_key = P.key;
    }
    return 0;
}

int fpt_cuda_autotune_batch(const struct FptRenderConfig *configs, const struct FptCudaSceneExt *exts, size_t count, uint32_t rounds,
                            struct FptCudaTuneResult *result, char *error, size_t error_len) {
    if (result) std::memset(result, 0, sizeof(*result));
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    BatchPlan P;
    if (!make_plan(configs, exts, count, P, error, error_len)) return 1;
    rounds = std::max<uint32_t>(std::min<uint32_t>(rounds, 15), 1);
    struct Cand { TuneChoice choice; std::vector<float> ms; };
    std::vector<Cand> cands;
    const uint32_t waves[3] = {0u, 1u << 20, 4u << 20};
    for (int v = 0; v < kVariantCount; ++v) cands.push_back({TuneChoice{v, 0u, 0u}, {}});
    for (int w = 1; w < 3; ++w)
        if (waves[w] < P.work) cands.push_back({TuneChoice{0, waves[w], 0u}, {}});
    for (uint32_t refill : {1u, 4u, 16u}) cands.push_back({TuneChoice{0, 0u, refill}, {}});
    // warm-up once per candidate, then interleaved timed rounds
    for (int r = -1; r < int(rounds); ++r)
        for (auto &cd : cands) {
            float ms = 0.0f;
            uint32_t launches = 0;
            double build_ms = 0.0;
            if (!render_plan(P, cd.choice, ms, launches, build_ms, error, error_len)) return 1;
            if (r >= 0) cd.ms.push_back(ms);
        }
    auto median = [](std::vector<float> v) {
        std::sort(v.begin(), v.end());
        return double(v[v.size() / 2]);
    };
    size_t best = 0;
    const double base = median(cands[0].ms);
    double best_ms = base;
    for (size_t i = 1; i < cands.size(); ++i) {
        const double m = median(cands[i].ms);
        if (m < best_ms && m < base * (1.0 - kTuneMargin)) { best_ms = m; best = i; }
    }
    tuned()[P.key] = cands[best].choice;
    if (result) {
        result->candidates = uint32_t(std::min<size_t>(cands.size(), 16));
        result->chosen = uint32_t(best);
        result->rounds = rounds;
        result->workload_key = P.key;
        for (size_t i = 0; i < cands.size() && i < 16; ++i) {
            const MarchVariant &V = kVariants[cands[i].choice.variant];
            cudaFuncAttributes fa{};
            cudaFuncGetAttributes(&fa, V.fn);
            result->tried[i].block_size = uint32_t(V.block);
            result->tried[i].registers = uint32_t(fa.numRegs);
            result->tried[i].wave_paths = wave_for(P, cands[i].choice.wave_paths);
            result->tried[i].refill = cands[i].choice.refill;
            result->tried[i].median_ms = median(cands[i].ms);
        }
    }
    return 0;
}

}  // extern "C"
