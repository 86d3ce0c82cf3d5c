// Instance cull + single-pass prefix sum, and the per-meshlet cull that
// writes the draw lists ("mesh shaders in compute").
//
// Reference passes: cull_instances / cull_instances_shadows
// (src/shaders/cull_instances.comp:7-56) appending into a prefix-sum sector
// with one 64-bit atomicAdd of {count:hi32, sum:lo32}
// (src/shaders/common/prefix_sum.glsl:17-30), and write_draw_calls /
// write_draw_calls_shadows (src/shaders/write_draw_calls.comp:7-117), which
// look up each candidate meshlet with an upper_bound over the inclusive sums
// (prefix_sum.glsl:33-46, util.glsl:42-59) and append visible meshlets with
// a 32-bit atomicAdd.
//
// GB300 design: the appends are order-preserving.  Each block owns one tile
// (claimed in order from a per-view counter), reduces its tile with warp
// scans, publishes the tile aggregate in one 64-bit status word and looks
// back over its predecessors' words (decoupled look-back) for its exclusive
// prefix.  The output order is therefore the canonical one -- instances
// ascending, then meshlets ascending -- and visible lists / visibility IDs are
// deterministic.  The sector keeps the reference layout and its final packed
// {count:hi32, sum:lo32} counter.
#pragma once

#include "lh_device.cuh"
#include "lh_internal.cuh"
#include "sphere_box.cuh"

namespace lh {
namespace {

__device__ __forceinline__ void st_status(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_status(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Decoupled look-back by one warp (every lane calls it; the result is the
// same on all): publish the tile aggregate, then read the status words of
// the 32 preceding tiles at once, lane i the (i + 1)-th predecessor.  When
// one of them holds an inclusive prefix, the nearest one ends the walk: the
// aggregates of the tiles after it and that prefix sum to the exclusive
// prefix; when none does (all 32 ready), their aggregates are added and the
// window moves 32 tiles back.  Words before tile 0 read as an inclusive 0.
// Publishes the tile's inclusive prefix.  The payloads add field-wise.
// Every wait is bounded (`limit` polls of the window); on expiry the status
// flag LH_FLAG_TIMEOUT is set and the missing predecessors count as zero (no
// hang, results flagged).
__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (uint32_t o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
__device__ __noinline__ uint64_t lookback_warp(uint64_t* status, uint32_t tile, uint64_t agg, uint32_t* flags,
                                               uint32_t limit = kSpinLimit) {
    const uint32_t lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) st_status(&status[0], kStatIncl | agg);
        return 0;
    }
    if (lane == 0) st_status(&status[tile], kStatAgg | agg);
    uint64_t excl = 0;
    int64_t base = (int64_t)tile - 1;  // the window's nearest predecessor
    uint32_t spins = 0;
    bool timed_out = false;
    for (;;) {
        const int64_t t = base - (int64_t)lane;
        const uint64_t s = t >= 0 ? ld_status(&status[t]) : kStatIncl;
        const uint32_t fl = (uint32_t)(s >> 62);
        const uint32_t incl = __ballot_sync(0xFFFFFFFFu, fl == 2u);
        const uint32_t not_ready = __ballot_sync(0xFFFFFFFFu, fl == 0u);
        const uint32_t first = incl ? (uint32_t)(__ffs(incl) - 1) : 31u;
        const uint32_t need = first == 31u ? 0xFFFFFFFFu : (2u << first) - 1u;  // lanes 0 .. first
        if (not_ready & need) {
            if (++spins < limit) {
                if (spins > 32) __nanosleep(spins > 1024 ? 256 : 32);
                continue;
            }
            timed_out = true;  // the missing words count as zero
        }
        excl += warp_sum_u64(lane <= first && fl != 0u ? (s & kPayloadMask) : 0ull);
        if (incl || timed_out) break;
        base -= 32;
        spins = 0;
    }
    if (lane == 0) {
        if (timed_out) atomicOr(&flags[kStFlags], LH_FLAG_TIMEOUT);
        st_status(&status[tile], kStatIncl | (excl + agg));
    }
    return excl;
}


// Radius of a ball of radius r after the linear part of `m` (columns 0..2):
// r times a bound of the largest singular value, sqrt of Gershgorin's bound
// on the eigenvalues of M^T M (exact for orthogonal columns, an upper bound
// for any matrix), widened by 2^-16 for the rounding of the float sums.
__device__ __forceinline__ float bounding_radius(const float4 (&c)[4], float r) {
    const float n0 = c[0].x * c[0].x + c[0].y * c[0].y + c[0].z * c[0].z;
    const float n1 = c[1].x * c[1].x + c[1].y * c[1].y + c[1].z * c[1].z;
    const float n2 = c[2].x * c[2].x + c[2].y * c[2].y + c[2].z * c[2].z;
    const float d01 = fabsf(c[0].x * c[1].x + c[0].y * c[1].y + c[0].z * c[1].z);
    const float d02 = fabsf(c[0].x * c[2].x + c[0].y * c[2].y + c[0].z * c[2].z);
    const float d12 = fabsf(c[1].x * c[2].x + c[1].y * c[2].y + c[1].z * c[2].z);
    const float lam = fmaxf(fmaxf(n0 + d01 + d02, n1 + d01 + d12), n2 + d02 + d12);
    return r * sqrtf(lam) * (1.0f + 1.0f / 65536.0f);
}

// The raster's record of a visible meshlet (the scene records it reads were
// loaded moments earlier by the same thread, so these loads mostly hit):
// the addresses of its vertex data, its world-space bounding sphere, and --
// in a visibility view with occlusion culling -- whether it is an occluder:
// opaque, with a projected sphere radius above f.occlusion_px pixels (or
// reaching the camera plane).  Occluders are appended to the view's
// occluder list (any order: the raster is order independent).
__device__ __forceinline__ RasterDraw raster_draw_of(const FrameDev& f, const ViewDev* vw, const Uniforms& u,
                                                     const lh_mat4& vp, MeshletReference ref, bool alpha,
                                                     uint32_t slot) {
    const Instance* inst = f.instances + ref.instance_index;
    const unsigned long long* mw = reinterpret_cast<const unsigned long long*>(__ldg(&inst->mesh_info_address));
    const uint64_t positions = __ldg(mw + 0), indices = __ldg(mw + 1), micro = __ldg(mw + 4), meshlets = __ldg(mw + 5);
    const uint32_t mflags = (uint32_t)((__ldg(mw + 6) >> 16) & 0xFFu);
    // Meshlet words at byte 44: triangle_offset, index_offset, counts
    const uint32_t* ml = reinterpret_cast<const uint32_t*>(reinterpret_cast<const Meshlet*>(meshlets) + ref.meshlet_index);
    const uint32_t tri_off = __ldg(ml + 11), idx_off = __ldg(ml + 12), counts = __ldg(ml + 13);
    RasterDraw r;
    r.positions = positions;
    r.indices = indices + (uint64_t)idx_off * ((mflags & MESH_INFO_FLAGS_32_BIT_INDICES) ? 4u : 2u);
    r.micro = micro + tri_off;
    r.instance = ref.instance_index;
    // counts = triangle_count | index_count << 8
    r.bits = ((counts >> 8) & 0xFFu) | ((counts & 0xFFu) << 8) | (mflags << 16);
    // world sphere: transform * centre, radius through the linear part
    float4 tc[4];
    const float4* tsrc = reinterpret_cast<const float4*>(inst);
#pragma unroll
    for (int c = 0; c < 4; c++) tc[c] = __ldg(tsrc + c);
    const float* mls = reinterpret_cast<const float*>(ml) + 7;  // Meshlet.bounding_sphere at byte 28
    const float bx = __ldg(mls), by = __ldg(mls + 1), bz = __ldg(mls + 2), br = __ldg(mls + 3);
    const float wx = ((tc[0].x * bx + tc[1].x * by) + tc[2].x * bz) + tc[3].x;
    const float wy = ((tc[0].y * bx + tc[1].y * by) + tc[2].y * bz) + tc[3].y;
    const float wz = ((tc[0].z * bx + tc[1].z * by) + tc[2].z * bz) + tc[3].z;
    // plus 8 ulps of the largest coordinate: the raster's float world
    // positions of the vertices, rounded like this centre, stay inside
    const float R = bounding_radius(tc, br) + fmaxf(fmaxf(fabsf(wx), fabsf(wy)), fabsf(wz)) * (1.0f / 1048576.0f);
    r.sphere[0] = wx;
    r.sphere[1] = wy;
    r.sphere[2] = wz;
    r.sphere[3] = R;
    // small views (probes): a meshlet whose sphere reaches no pixel centre
    // is common there, and the raster skips it before its vertices (in
    // large views the test would cost the cull more than it saves)
    if (vw->width * vw->height <= kNoCentreTestPixels && sphere_misses_centres(vp, wx, wy, wz, R, vw->width, vw->height)) {
        r.bits |= kDrawNoCentre;
        return r;
    }
    if (f.occlusion_px && !alpha && vw->kind == kViewVisibility && vw->lists) {
        const lh_mat4& pv = u.combined_perspective_view;
        const float w = ((pv.cols[0].w * wx + pv.cols[1].w * wy) + pv.cols[2].w * wz) + pv.cols[3].w;
        const float focal_px = fabsf(u.perspective.cols[1].y) * 0.5f * (float)vw->height;
        if (!(w > R) || R * focal_px > (float)f.occlusion_px * (w - R)) {
            r.bits |= kDrawOccluder;
            const uint32_t pos = atomicAdd(&vw->claim[kClaimOccluders], 1u);
            if (pos < f.max_draws) vw->lists[pos] = slot;
        }
    }
    return r;
}

// Fields of a MeshInfo the cull needs (loaded as aligned 8-byte words).
struct MeshInfoCull {
    uint64_t meshlets;
    uint32_t num_meshlets;
    uint32_t flags;
    lh_vec4 bounding_sphere;
};
__device__ __forceinline__ MeshInfoCull load_mesh_info(const MeshInfo* mi) {
    const unsigned long long* w = reinterpret_cast<const unsigned long long*>(mi);
    unsigned long long w5 = __ldg(w + 5), w6 = __ldg(w + 6), w7 = __ldg(w + 7);
    uint32_t w8 = __ldg(reinterpret_cast<const uint32_t*>(mi) + 16);
    MeshInfoCull r;
    r.meshlets = w5;
    r.num_meshlets = (uint32_t)(w6 & 0xFFFFu);
    r.flags = (uint32_t)((w6 >> 16) & 0xFFu);
    r.bounding_sphere.x = __uint_as_float((uint32_t)(w6 >> 32));
    r.bounding_sphere.y = __uint_as_float((uint32_t)w7);
    r.bounding_sphere.z = __uint_as_float((uint32_t)(w7 >> 32));
    r.bounding_sphere.w = __uint_as_float(w8);
    return r;
}

// Copy a struct of `bytes` (multiple of 8) into shared memory.
__device__ __forceinline__ void copy_to_smem(void* dst, const void* src, uint32_t bytes) {
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
    for (uint32_t i = threadIdx.x; i < bytes / 8; i += blockDim.x) d[i] = s[i];
}

// Inclusive warp scan of a 64-bit additive payload.
__device__ __forceinline__ uint64_t warp_incl_scan(uint64_t v) {
    const uint32_t lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t n = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= (uint32_t)o) v += n;
    }
    return v;
}

constexpr uint64_t kSum40 = (1ull << 40) - 1;

// ---------------------------------------------------------------- instance cull
// One tile (kInstTile instances) of view `view`; the tile is claimed in order
// from the view's counter, so blocks only ever wait on tiles claimed before
// theirs.  `n_tiles` = tiles of the view (the last one writes the counter).
__device__ void phase_cull_instances_tile(const FrameDev& f, uint32_t view, uint32_t n_tiles) {
    __shared__ __align__(16) Uniforms s_u;
    __shared__ __align__(16) MiscStorage s_m;
    __shared__ uint64_t s_warp[kInstTile / 32];
    __shared__ uint64_t s_excl;
    __shared__ uint32_t s_tile;
    const ViewDev* vw = f.views + view;
    const uint32_t kind = vw->kind, cascade = vw->cascade;
    if (threadIdx.x == 0) s_tile = atomicAdd(&vw->claim[0], 1u);
    if (kind == kViewVisibility)
        copy_to_smem(&s_u, vw->uniforms, sizeof(Uniforms));
    else
        copy_to_smem(&s_m, f.misc, sizeof(MiscStorage));
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t i = tile * kInstTile + threadIdx.x;
    bool keep = false;
    uint32_t nm = 0;
    if (i < f.n_instances) {
        InstanceBits ib;
        load_instance(f.instances + i, ib);
        MeshInfoCull mi = load_mesh_info(mesh_info_of(&ib.inst));
        nm = mi.num_meshlets;
        keep = kind == kViewVisibility ? !cull_bounding_sphere(s_u, ib.inst.transform, mi.bounding_sphere)
                                       : !cull_bounding_sphere_shadows(s_m, ib.inst.transform, mi.bounding_sphere, cascade);
    }
    const uint64_t pay = keep ? ((1ull << 40) | nm) : 0ull;
    uint64_t incl = warp_incl_scan(pay);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint64_t run = 0;
        if (lane == 0)
            for (uint32_t w = 0; w < kInstTile / 32; w++) {
                uint64_t t = s_warp[w];
                s_warp[w] = run;
                run += t;
            }
        run = __shfl_sync(0xFFFFFFFFu, run, 0);
        const uint64_t excl = lookback_warp(vw->inst_status, tile, run, f.status);
        if (lane == 0) s_excl = excl;
        if (lane == 0 && tile == n_tiles - 1) {
            uint64_t total = excl + run;
            uint64_t count = total >> 40;
            *reinterpret_cast<unsigned long long*>(vw->sector) = (count << 32) | (uint32_t)(total & kSum40);
            if (count > f.max_instances) atomicOr(&f.status[kStFlags], LH_FLAG_INSTANCE_OVERFLOW);
        }
    }
    __syncthreads();
    if (keep) {
        uint64_t before = s_excl + s_warp[warp] + incl - pay;
        uint32_t pos = (uint32_t)(before >> 40);
        if (pos < f.max_instances) {
            PrefixSumValue v;
            v.index = i;
            v.sum = (uint32_t)(before & kSum40) + nm;
            reinterpret_cast<PrefixSumValue*>(vw->sector + 8)[pos] = v;
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------- meshlet cull
__device__ __forceinline__ uint32_t upper_bound(const PrefixSumValue* v, uint32_t count, uint32_t target) {
    uint32_t first = 0;
    while (count > 0) {
        uint32_t step = count / 2, cur = first + step;
        bool greater = target >= v[cur].sum;
        first = greater ? cur + 1 : first;
        count = greater ? count - (step + 1) : step;
    }
    return first;
}

// upper_bound by one warp: 32 probes per step (log32 of the count dependent
// loads instead of log2).  The entries' sums do not decrease, so the probes
// with sum <= target form a prefix of the lanes.
__device__ __forceinline__ uint32_t upper_bound_warp(const PrefixSumValue* v, uint32_t count, uint32_t target,
                                                     uint32_t lane) {
    uint32_t lo = 0, hi = count;  // the answer lies in [lo, hi]
    for (;;) {
        const uint32_t span = hi - lo;
        const uint32_t step = span <= 32u ? 1u : (span + 31u) / 32u;
        const uint32_t p = lo + lane * step;
        const bool le = p < hi && v[p].sum <= target;
        const uint32_t k = __popc(__ballot_sync(0xFFFFFFFFu, le));
        if (step == 1u) return lo + k;
        const uint32_t nlo = k ? lo + (k - 1u) * step + 1u : lo;
        const uint32_t nhi = (k < 32u && lo + k * step < hi) ? lo + k * step : hi;
        lo = nlo;
        hi = nhi;
    }
}

// Candidate count of a view's sector (an overflowing sector holds only its
// first max_instances entries).
__device__ __forceinline__ void sector_extent(const FrameDev& f, const ViewDev* vw, uint32_t& count, uint32_t& total) {
    const PrefixSumValue* values = reinterpret_cast<const PrefixSumValue*>(vw->sector + 8);
    const unsigned long long counter = *reinterpret_cast<volatile unsigned long long*>(vw->sector);
    count = (uint32_t)(counter >> 32);
    total = (uint32_t)counter;
    if (count > f.max_instances) {
        count = f.max_instances;
        total = count ? values[count - 1].sum : 0;
    }
}

// Meshlet cull of views [view_begin, view_begin + n_views): every block
// claims (view, tile) pairs from one counter (`claim_word`), tiles of
// kMlTile candidates in order within each view.  Persistent: returns when the
// claims are exhausted.
__device__ void phase_cull_meshlets(const FrameDev& f, uint32_t view_begin, uint32_t n_views, uint32_t* claim_word) {
    __shared__ __align__(16) Uniforms s_u;
    __shared__ __align__(16) MiscStorage s_m;
    __shared__ PrefixSumValue s_entries[kMlTile];
    __shared__ uint32_t s_cnt[2][kMlItems * (kMlThreads / 32)];
    __shared__ uint32_t s_tile, s_view, s_eab[2], s_tot[2], s_loaded_view;
    __shared__ uint32_t s_tile_off[kMaxViews + 1];
    __shared__ uint64_t s_excl;
    const uint32_t md = f.max_draws;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t v = 0; v < n_views; v++) {
            const ViewDev* vw = f.views + view_begin + v;
            uint32_t count, total;
            sector_extent(f, vw, count, total);
            uint32_t n_tiles = (uint32_t)(((uint64_t)total + kMlTile - 1) / kMlTile);
            if (n_tiles > vw->ml_tile_cap) {
                atomicOr(&f.status[kStFlags], LH_FLAG_DRAW_OVERFLOW);
                n_tiles = vw->ml_tile_cap;
            }
            s_tile_off[v] = run;
            run += n_tiles;
        }
        s_tile_off[n_views] = run;
        s_loaded_view = 0xFFFFFFFFu;
    }
    __syncthreads();
    const uint32_t all_tiles = s_tile_off[n_views];
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t c = atomicAdd(claim_word, 1u);
            uint32_t v = 0;
            if (c < all_tiles)
                while (c >= s_tile_off[v + 1]) v++;
            s_view = v;
            s_tile = c;
        }
        __syncthreads();
        if (s_tile >= all_tiles) break;
        const uint32_t v = s_view;
        const uint32_t tile = s_tile - s_tile_off[v];
        const ViewDev* vw = f.views + view_begin + v;
        const uint32_t kind = vw->kind, cascade = vw->cascade;
        if (s_loaded_view != v) {
            copy_to_smem(&s_u, vw->uniforms, sizeof(Uniforms));
            if (kind == kViewShadow) copy_to_smem(&s_m, f.misc, sizeof(MiscStorage));
        }
        const PrefixSumValue* values = reinterpret_cast<const PrefixSumValue*>(vw->sector + 8);
        uint32_t count, total;
        sector_extent(f, vw, count, total);
        const uint32_t n_tiles = s_tile_off[v + 1] - s_tile_off[v];
        const uint32_t t0 = tile * kMlTile, t1 = min(total, t0 + kMlTile);
        // the tile's first and last entries, one warp each
        if (warp < 2) {
            const uint32_t e = upper_bound_warp(values, count, warp == 0 ? t0 : t1 - 1, lane);
            if (lane == 0) s_eab[warp] = e;
        }
        __syncthreads();
        const uint32_t ea = s_eab[0], ne = s_eab[1] - s_eab[0] + 1;
        const bool smem_entries = ne <= kMlTile;
        if (smem_entries)
            for (uint32_t j = threadIdx.x; j < ne; j += kMlThreads) s_entries[j] = values[ea + j];
        // every thread has passed the s_loaded_view test above (barrier), and
        // none reads it again before the next claim's barrier
        if (threadIdx.x == 0) s_loaded_view = v;
        __syncthreads();

        uint32_t cls_bits = 0;  // 2 bits per item: 1 opaque, 2 alpha clip
        MeshletReference refs[kMlItems];
        uint32_t tris[(kMlItems + 3) / 4];  // triangle count per item, 8 bits each
#pragma unroll
        for (uint32_t k = 0; k < (kMlItems + 3) / 4; k++) tris[k] = 0;
#pragma unroll
        for (uint32_t k = 0; k < kMlItems; k++) {
            const uint32_t c = t0 + k * kMlThreads + threadIdx.x;
            refs[k].instance_index = 0;
            refs[k].meshlet_index = 0;
            if (c < t1) {
                PrefixSumValue r;
                if (smem_entries) {
                    uint32_t j = upper_bound(s_entries, ne, c);
                    r = s_entries[min(j, ne - 1)];
                } else {
                    r = values[min(upper_bound(values, count, c), count - 1)];
                }
                InstanceBits ib;
                load_instance(f.instances + r.index, ib);
                const MeshInfo* mip = mesh_info_of(&ib.inst);
                MeshInfoCull mi = load_mesh_info(mip);
                uint32_t local = c - (r.sum - mi.num_meshlets);
                refs[k].instance_index = r.index;
                refs[k].meshlet_index = (uint16_t)local;
                MeshletBits mb;
                load_meshlet(reinterpret_cast<const Meshlet*>(mi.meshlets) + (uint16_t)local, mb);
                tris[k / 4] |= (uint32_t)mb.m.triangle_count << (8 * (k % 4));
                const bool alpha = (mi.flags & MESH_INFO_FLAGS_ALPHA_CLIP) != 0;
                bool vis;
                if (kind == kViewVisibility)
                    vis = !cull_bounding_sphere(s_u, ib.inst.transform, mb.m.bounding_sphere) &&
                          (alpha || !cull_cone_perspective(s_u, &ib.inst, ib.inst.transform, mb.m));
                else
                    vis = !cull_bounding_sphere_shadows(s_m, ib.inst.transform, mb.m.bounding_sphere, cascade) &&
                          (alpha || !cull_cone_orthographic(s_u, &ib.inst, mb.m));
                if (vis) cls_bits |= (alpha ? 2u : 1u) << (2 * k);
            }
        }
        // Ordered compaction: counts per (item k, warp), k-major.
        uint32_t bal_op[kMlItems], bal_al[kMlItems];
#pragma unroll
        for (uint32_t k = 0; k < kMlItems; k++) {
            uint32_t cl = (cls_bits >> (2 * k)) & 3u;
            bal_op[k] = __ballot_sync(0xFFFFFFFFu, cl == 1u);
            bal_al[k] = __ballot_sync(0xFFFFFFFFu, cl == 2u);
            if (lane == 0) {
                s_cnt[0][k * (kMlThreads / 32) + warp] = __popc(bal_op[k]);
                s_cnt[1][k * (kMlThreads / 32) + warp] = __popc(bal_al[k]);
            }
        }
        __syncthreads();
        if (warp == 0) {
            // exclusive scan of N counts per class: PER consecutive ones on
            // each of the first LANES lanes
            constexpr uint32_t N = kMlItems * (kMlThreads / 32);
            constexpr uint32_t PER = N >= 32 ? N / 32 : 1;
            constexpr uint32_t LANES = N / PER;
            static_assert(N % PER == 0 && LANES <= 32 && PER <= 4, "scan layout");
#pragma unroll
            for (int cl = 0; cl < 2; cl++) {
                uint32_t c[PER], s = 0;
#pragma unroll
                for (uint32_t i = 0; i < PER; i++) {
                    c[i] = lane < LANES ? s_cnt[cl][PER * lane + i] : 0u;
                    s += c[i];
                }
                uint32_t incl = s;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                    if (lane >= (uint32_t)o) incl += n;
                }
                uint32_t ex = incl - s;
#pragma unroll
                for (uint32_t i = 0; i < PER; i++) {
                    if (lane < LANES) s_cnt[cl][PER * lane + i] = ex;
                    ex += c[i];
                }
                if (lane == 31) s_tot[cl] = incl;
            }
            __syncwarp();
            const uint64_t agg = ((uint64_t)s_tot[0] << 31) | (uint64_t)s_tot[1];
            const uint64_t excl = lookback_warp(vw->ml_status, tile, agg, f.status);
            if (lane == 0) {
                s_excl = excl;
                if (tile == n_tiles - 1) {
                    uint64_t tot = excl + agg;
                    uint32_t nop = (uint32_t)(tot >> 31), nal = (uint32_t)(tot & 0x7FFFFFFFu);
                    uint32_t* draw_counts = reinterpret_cast<uint32_t*>(vw->draws);
                    draw_counts[0] = nop;
                    draw_counts[1] = nal;
                    if (nop > md || nal > md) atomicOr(&f.status[kStFlags], LH_FLAG_DRAW_OVERFLOW);
                }
            }
        }
        __syncthreads();
        const uint32_t ex_op = (uint32_t)(s_excl >> 31), ex_al = (uint32_t)(s_excl & 0x7FFFFFFFu);
        const uint32_t lt = (1u << lane) - 1u;
        MeshletReference* out_refs = vw->refs;
        DrawIndirectCommand* draws = reinterpret_cast<DrawIndirectCommand*>(vw->draws + 8);
#pragma unroll
        for (uint32_t k = 0; k < kMlItems; k++) {
            uint32_t cl = (cls_bits >> (2 * k)) & 3u;
            if (!cl) continue;
            uint32_t pos, slot;
            if (cl == 1u) {
                pos = ex_op + s_cnt[0][k * (kMlThreads / 32) + warp] + __popc(bal_op[k] & lt);
                slot = pos;
            } else {
                pos = ex_al + s_cnt[1][k * (kMlThreads / 32) + warp] + __popc(bal_al[k] & lt);
                slot = md + pos;
            }
            if (pos >= md) continue;
            DrawIndirectCommand dc;
            dc.vertexCount = ((tris[k / 4] >> (8 * (k % 4))) & 0xFFu) * 3u;
            dc.instanceCount = 1;
            dc.firstVertex = 0;
            dc.firstInstance = vw->section_base + slot;
            draws[slot] = dc;
            out_refs[slot] = refs[k];
            vw->rdraws[slot] = raster_draw_of(f, vw, s_u, kind == kViewVisibility ? s_u.combined_perspective_view
                                                                                  : s_m.shadow_matrices[cascade],
                                              refs[k], cl == 2u, slot);
        }
        __syncthreads();
    }
    __syncthreads();
}

}  // namespace
}  // namespace lh
