// voxel_dda.cuh -- exact grid DDA over sparse voxel bricks (device code).
//
// Restates the traversal contract of shaders/Shaders.metal:4091-4190 and
// traceVoxel (4492-4612): slab clip, direction-aware half-open start cell,
// per-axis next_t / delta_t, ties crossing several axes at once, and the
// next-representable-float step when a boundary does not advance t.  This
// header is compiled only into voxel.cu, which is built with -fmad=false:
// every operation rounds separately in source order, so cell sequences and
// hit distances are bit-identical to the CPU path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpt {
namespace vox {

constexpr float kInfF = 1.0e20f;   // the reference's `inf` constant

struct Grid {
    float bmin[3], bmax[3], cs[3];
    uint32_t res;
    uint32_t brick_shift;          // log2(brick size): 2 (4^3) or 3 (8^3)
    uint32_t brick_grid;           // bricks per axis
    uint32_t storage;              // 0 dense, 1 sparse bricks (reference cells), 4 occupancy bricks
    const uint32_t *table;         // brick table: 0 = empty, else compact brick index + 1
    const uint8_t *occ;            // occupancy bricks: brick_size^3 bytes per brick
    const uint64_t *mask;          // occupancy bricks: brick_size^3 / 64 words per brick (derived index)
    const uint32_t *cells;         // reference cells: 3 words per cell (colour|bit31, properties, emission)
};

__device__ __forceinline__ float axis(const float3 &v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void set_axis(float3 &v, int a, float x) { if (a == 0) v.x = x; else if (a == 1) v.y = x; else v.z = x; }
__device__ __forceinline__ int iaxis(const int3 &v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void set_iaxis(int3 &v, int a, int x) { if (a == 0) v.x = x; else if (a == 1) v.y = x; else v.z = x; }

// voxelRayAabb (:4107-4136)
__device__ __forceinline__ bool ray_aabb(float3 o, float3 d, const float *bmin, const float *bmax, float &near_t, float &far_t,
                                         float3 &entry_normal) {
    near_t = -kInfF;
    far_t = kInfF;
    entry_normal = make_float3(0.f, 0.f, 0.f);
    for (int a = 0; a < 3; ++a) {
        float da = axis(d, a), oa = axis(o, a);
        if (da == 0.0f) {
            if (oa < bmin[a] || oa > bmax[a]) return false;
            continue;
        }
        float t0 = (bmin[a] - oa) / da;
        float t1 = (bmax[a] - oa) / da;
        float an = fminf(t0, t1), af = fmaxf(t0, t1);
        if (an > near_t) {
            near_t = an;
            entry_normal = make_float3(0.f, 0.f, 0.f);
            set_axis(entry_normal, a, da > 0.0f ? -1.0f : 1.0f);
        }
        far_t = fminf(far_t, af);
        if (near_t > far_t) return false;
    }
    float entry_t = fmaxf(near_t, 0.0f);
    return isfinite(entry_t) && isfinite(far_t) && far_t >= entry_t;
}

// voxelCellCoordinate (:4141-4158)
__device__ __forceinline__ bool cell_coordinate(float3 p, float3 d, const Grid &g, int3 &cell) {
    for (int a = 0; a < 3; ++a) {
        float pa = axis(p, a);
        if (pa < g.bmin[a] || pa > g.bmax[a]) return false;
    }
    for (int a = 0; a < 3; ++a) {
        float pa = axis(p, a), da = axis(d, a);
        if ((da < 0.0f && pa <= g.bmin[a]) || (da > 0.0f && pa >= g.bmax[a])) return false;
    }
    int r = int(g.res);
    for (int a = 0; a < 3; ++a) {
        float gp = (axis(p, a) - g.bmin[a]) / g.cs[a];
        float fl = floorf(gp);
        int c = int(fl) - ((axis(d, a) < 0.0f && gp == fl) ? 1 : 0);
        c = min(c, r - 1);
        if (c < 0 || c >= r) return false;
        set_iaxis(cell, a, c);
    }
    return true;
}

// voxelNextPositiveFloat (:4163-4167)
__device__ __forceinline__ float next_positive_float(float v) {
    if (!isfinite(v) || v < 0.0f) return kInfF;
    if (v == 0.0f) return __uint_as_float(1u);
    return __uint_as_float(__float_as_uint(v) + 1u);
}

// voxelAdvanceDda (:4169-4190)
__device__ __forceinline__ bool advance(int3 &cell, int3 step, float3 &next_t, float3 delta_t, float &entry_t, float3 &entry_normal) {
    float bt = fminf(next_t.x, fminf(next_t.y, next_t.z));
    if (!isfinite(bt)) return false;
    bool cx = next_t.x == bt, cy = next_t.y == bt, cz = next_t.z == bt;
    float ne = bt;
    if (!(ne > entry_t)) {
        ne = next_positive_float(entry_t);
        if (!isfinite(ne) || !(ne > entry_t)) return false;
    }
    entry_t = ne;
    entry_normal = make_float3(0.f, 0.f, 0.f);
    int na = cx ? 0 : (cy ? 1 : 2);
    set_axis(entry_normal, na, iaxis(step, na) > 0 ? -1.0f : 1.0f);
    if (cx) { cell.x += step.x; next_t.x = next_t.x + delta_t.x; }
    if (cy) { cell.y += step.y; next_t.y = next_t.y + delta_t.y; }
    if (cz) { cell.z += step.z; next_t.z = next_t.z + delta_t.z; }
    return true;
}

struct Hit {
    bool hit;
    float t, exit_t;
    int3 cell;
    float3 normal;
    uint32_t steps;
    uint32_t brick_fetches;
};

// Occupancy of one cell (storage formats of the build).
__device__ __forceinline__ bool occupied(const Grid &g, int3 c, uint32_t &payload_index, uint32_t &fetches) {
    uint32_t x = uint32_t(c.x), y = uint32_t(c.y), z = uint32_t(c.z);
    if (g.storage == 0u) {
        payload_index = x + y * g.res + z * g.res * g.res;
        return (g.cells[size_t(payload_index) * 3] & 0x80000000u) != 0u;
    }
    uint32_t sh = g.brick_shift, bs = 1u << sh, m = bs - 1u;
    uint32_t b = (x >> sh) + (y >> sh) * g.brick_grid + (z >> sh) * g.brick_grid * g.brick_grid;
    uint32_t page = __ldg(g.table + b);
    ++fetches;
    if (page == 0u) return false;
    uint32_t local = (x & m) + (y & m) * bs + (z & m) * bs * bs;
    payload_index = (page - 1u) * bs * bs * bs + local;
    if (g.storage == 4u) {
        uint64_t w = __ldg(reinterpret_cast<const unsigned long long *>(g.mask) + (payload_index >> 6));
        return (w >> (payload_index & 63u)) & 1ull;
    }
    return (g.cells[size_t(payload_index) * 3] & 0x80000000u) != 0u;
}

// traceVoxel (:4492-4612) without leaf refinement.  When `seq` is given,
// every visited cell's linear index is recorded (up to seq_cap entries).
__device__ __forceinline__ Hit trace(const Grid &g, float3 o, float3 d, uint32_t *seq, uint32_t seq_cap, uint32_t *seq_len,
                                     uint32_t *payload_out) {
    Hit h;
    h.hit = false; h.t = kInfF; h.exit_t = kInfF; h.cell = make_int3(0, 0, 0); h.normal = make_float3(0.f, 0.f, 0.f);
    h.steps = 0; h.brick_fetches = 0;
    if (seq_len) *seq_len = 0;
    float near_t, far_t;
    float3 en;
    if (!ray_aabb(o, d, g.bmin, g.bmax, near_t, far_t, en)) return h;
    float entry_t = fmaxf(near_t, 0.0f);
    float3 start = make_float3(fminf(fmaxf(o.x + d.x * entry_t, g.bmin[0]), g.bmax[0]),
                               fminf(fmaxf(o.y + d.y * entry_t, g.bmin[1]), g.bmax[1]),
                               fminf(fmaxf(o.z + d.z * entry_t, g.bmin[2]), g.bmax[2]));
    int3 cell;
    if (!cell_coordinate(start, d, g, cell)) return h;
    int3 step = make_int3(0, 0, 0);
    float3 next_t = make_float3(kInfF, kInfF, kInfF), delta_t = make_float3(kInfF, kInfF, kInfF);
    for (int a = 0; a < 3; ++a) {
        float da = axis(d, a), oa = axis(o, a);
        float nt = kInfF, dt = kInfF;
        if (da > 0.0f) {
            set_iaxis(step, a, 1);
            float boundary = g.bmin[a] + float(iaxis(cell, a) + 1) * g.cs[a];
            nt = (boundary - oa) / da;
            dt = g.cs[a] / da;
        } else if (da < 0.0f) {
            set_iaxis(step, a, -1);
            float boundary = g.bmin[a] + float(iaxis(cell, a)) * g.cs[a];
            nt = (boundary - oa) / da;
            dt = -g.cs[a] / da;
        }
        if (!isfinite(nt) || !isfinite(dt)) { nt = kInfF; dt = kInfF; }
        set_axis(next_t, a, nt);
        set_axis(delta_t, a, dt);
    }
    const int r = int(g.res);
    const uint32_t max_steps = g.res * 3u + 3u;
    for (uint32_t s = 0; s < max_steps && entry_t <= far_t; ++s) {
        if (cell.x < 0 || cell.y < 0 || cell.z < 0 || cell.x >= r || cell.y >= r || cell.z >= r) break;
        if (seq && seq_len) {
            if (*seq_len < seq_cap) seq[*seq_len] = uint32_t(cell.x) + uint32_t(cell.y) * g.res + uint32_t(cell.z) * g.res * g.res;
            *seq_len += 1;
        }
        uint32_t payload = 0;
        if (occupied(g, cell, payload, h.brick_fetches)) {
            h.hit = true;
            h.t = entry_t;
            h.exit_t = fminf(next_t.x, fminf(next_t.y, next_t.z));
            h.cell = cell;
            h.normal = en;
            h.steps = s + 1;
            if (payload_out) *payload_out = payload;
            return h;
        }
        if (!advance(cell, step, next_t, delta_t, entry_t, en)) break;
    }
    return h;
}

// trace() specialised for occupancy bricks (8^3 cells, bit mask per brick)
// and for the render: one loop iteration per visited cell for every lane, so
// a warp's lanes stay in step (per-lane brick caching and per-lane inner
// loops over empty bricks were measured slower: whichever lane enters a new
// brick or leaves an empty one makes the whole warp run that code on most
// trips).  Per cell: the brick-table word (shift arithmetic, read-only
// cache), for an occupied brick one mask word, and the advance without the
// entry-normal writes -- the face normal is rebuilt at the hit from the axis
// crossed last.  Cells, entry distance, normal and step count equal trace()'s.
__device__ __forceinline__ Hit trace_bricks(const Grid &g, float3 o, float3 d) {
    Hit h;
    h.hit = false; h.t = kInfF; h.exit_t = kInfF; h.cell = make_int3(0, 0, 0); h.normal = make_float3(0.f, 0.f, 0.f);
    h.steps = 0; h.brick_fetches = 0;
    float near_t, far_t;
    float3 en;
    if (!ray_aabb(o, d, g.bmin, g.bmax, near_t, far_t, en)) return h;
    float entry_t = fmaxf(near_t, 0.0f);
    float3 start = make_float3(fminf(fmaxf(o.x + d.x * entry_t, g.bmin[0]), g.bmax[0]),
                               fminf(fmaxf(o.y + d.y * entry_t, g.bmin[1]), g.bmax[1]),
                               fminf(fmaxf(o.z + d.z * entry_t, g.bmin[2]), g.bmax[2]));
    int3 cell;
    if (!cell_coordinate(start, d, g, cell)) return h;
    int3 step = make_int3(0, 0, 0);
    float3 next_t = make_float3(kInfF, kInfF, kInfF), delta_t = make_float3(kInfF, kInfF, kInfF);
    for (int a = 0; a < 3; ++a) {
        float da = axis(d, a), oa = axis(o, a);
        float nt = kInfF, dt = kInfF;
        if (da > 0.0f) {
            set_iaxis(step, a, 1);
            float boundary = g.bmin[a] + float(iaxis(cell, a) + 1) * g.cs[a];
            nt = (boundary - oa) / da;
            dt = g.cs[a] / da;
        } else if (da < 0.0f) {
            set_iaxis(step, a, -1);
            float boundary = g.bmin[a] + float(iaxis(cell, a)) * g.cs[a];
            nt = (boundary - oa) / da;
            dt = -g.cs[a] / da;
        }
        if (!isfinite(nt) || !isfinite(dt)) { nt = kInfF; dt = kInfF; }
        set_axis(next_t, a, nt);
        set_axis(delta_t, a, dt);
    }
    int last_axis = -1;   // axis crossed by the last advance (-1: none yet, the normal is the box entry face)
    const int r = int(g.res);
    const uint32_t max_steps = g.res * 3u + 3u;
    const uint32_t bg = g.brick_grid;
    const unsigned long long *mask = reinterpret_cast<const unsigned long long *>(g.mask);
    for (uint32_t s = 0; s < max_steps && entry_t <= far_t; ++s) {
        if (cell.x < 0 || cell.y < 0 || cell.z < 0 || cell.x >= r || cell.y >= r || cell.z >= r) break;
        const uint32_t x = uint32_t(cell.x), y = uint32_t(cell.y), z = uint32_t(cell.z);
        const uint32_t page = __ldg(g.table + (x >> 3) + ((y >> 3) + (z >> 3) * bg) * bg);
        if (page != 0u && ((__ldg(mask + size_t(page - 1u) * 8u + (z & 7u)) >> ((x & 7u) + 8u * (y & 7u))) & 1ull)) {
            h.hit = true;
            h.t = entry_t;
            h.exit_t = fminf(next_t.x, fminf(next_t.y, next_t.z));
            h.cell = cell;
            if (last_axis >= 0) {
                const int st = last_axis == 0 ? step.x : (last_axis == 1 ? step.y : step.z);
                const float nv = st > 0 ? -1.0f : 1.0f;
                h.normal = make_float3(last_axis == 0 ? nv : 0.0f, last_axis == 1 ? nv : 0.0f, last_axis == 2 ? nv : 0.0f);
            } else {
                h.normal = en;
            }
            h.steps = s + 1;
            return h;
        }
        const float bt = fminf(next_t.x, fminf(next_t.y, next_t.z));
        if (!isfinite(bt)) break;
        const bool cx = next_t.x == bt, cy = next_t.y == bt, cz = next_t.z == bt;
        float ne = bt;
        if (!(ne > entry_t)) {
            ne = next_positive_float(entry_t);
            if (!isfinite(ne) || !(ne > entry_t)) break;
        }
        entry_t = ne;
        last_axis = cx ? 0 : (cy ? 1 : 2);
        if (cx) { cell.x += step.x; next_t.x = next_t.x + delta_t.x; }
        if (cy) { cell.y += step.y; next_t.y = next_t.y + delta_t.y; }
        if (cz) { cell.z += step.z; next_t.z = next_t.z + delta_t.z; }
    }
    return h;
}

}  // namespace vox
}  // namespace fpt
