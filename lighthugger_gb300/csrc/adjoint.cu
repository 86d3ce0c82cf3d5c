// Backward of the lighting resolve (render_geometry.comp:70-266) with the
// visibility held fixed: one thread per pixel recomputes the forward inputs
// from the visibility buffer (triangle, vertices, cascade, compare results)
// and runs the hand-written reverse pass of shade.cuh, then adds the
// gradients into the caller's buffers.  Targets every lane of a warp shares
// (light direction / colour, a material's base-colour factor) are summed
// across the warp first, so they take one atomic per warp.
#include <algorithm>

#include "frame_phases.cuh"
#include "shade.cuh"
#include "tma.cuh"

namespace lh {
namespace {

using shade::Bilinear;
using shade::PixelGrad;
using shade::PixelParams;
using shade::v2;
using shade::v3;

struct DeviceSampler {
    const FrameDev* f;
    __device__ Bilinear<float> sample(uint32_t index, v2<float> uv) const {
        Bilinear<float> s;
        s.index = index;
        if (index >= f->n_textures) {
            for (int c = 0; c < 4; c++) s.t00[c] = s.t10[c] = s.t01[c] = s.t11[c] = 0.0f;
            s.a = s.b = 0.0f;
            s.size_u = s.size_v = 0.0f;
            s.i0 = s.i1 = s.j0 = s.j1 = 0;
            return s;
        }
        const lh_texture t = f->textures[index];
        const float4* tex = f->tex_linear[index];
        float u = uv.x * (float)t.width - 0.5f, v = uv.y * (float)t.height - 0.5f;
        if (!(fabsf(u) < 1e9f)) u = 0.0f;
        if (!(fabsf(v) < 1e9f)) v = 0.0f;
        float fu = floorf(u), fv = floorf(v);
        s.a = u - fu;
        s.b = v - fv;
        const int32_t i0 = (int32_t)fu, j0 = (int32_t)fv;
        const int32_t W = (int32_t)t.width, H = (int32_t)t.height;
        s.i0 = wrap_texel(i0, W);
        s.i1 = wrap_texel(i0 + 1, W);
        s.j0 = wrap_texel(j0, H);
        s.j1 = wrap_texel(j0 + 1, H);
        s.size_u = (float)t.width;
        s.size_v = (float)t.height;
        auto texel = [&](int32_t i, int32_t j, float* o) {
            const float4 p = __ldg(tex + ((size_t)j * W + i));
            o[0] = p.x;
            o[1] = p.y;
            o[2] = p.z;
            o[3] = p.w;
        };
        texel(s.i0, s.j0, s.t00);
        texel(s.i1, s.j0, s.t10);
        texel(s.i0, s.j1, s.t01);
        texel(s.i1, s.j1, s.t11);
        return s;
    }
    __device__ float shadow_cmp(uint32_t layer, int32_t i, int32_t j, float ref) const {
        const int32_t S = (int32_t)f->shadow_size;
        i = i < 0 ? 0 : (i > S - 1 ? S - 1 : i);
        j = j < 0 ? 0 : (j > S - 1 ? S - 1 : j);
        return ref < __ldg(f->shadow_maps + ((size_t)layer * S + j) * S + i) ? 1.0f : 0.0f;
    }
};

constexpr uint32_t kFull = 0xFFFFFFFFu;
// Launch shape: tiles of 32 x ROWS pixels (ROWS = 4, 8 or 16, chosen at run
// time through lh_tuning.backward_rows), one warp per row, and the threads
// per SM the register budget is cut for (LH_BWD_MIN_BLOCKS blocks of 8 rows:
// 512 threads, 128 registers a thread, at every ROWS).
#ifndef LH_BWD_MIN_BLOCKS
#define LH_BWD_MIN_BLOCKS 2
#endif
constexpr uint32_t kCacheSlots = 256;     // shared-memory accumulators of hot gradient addresses
constexpr uint32_t kSmallTexture = 64;    // textures of at most this many texels go through them

// Fixed inputs of a pixel for shade.cuh whose matrices are read from
// memory at each use -- PV and the cascades' UVS from the block's shared
// copies, the instance's normal transform from global memory -- rather
// than held in registers through the whole pixel.  `pv3` / `uvs3` point at
// the column 3 in use (absolute for the decisions, camera-relative after).
__device__ __forceinline__ float lds_f32(const float* p) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(smem_u32(p)));
    return v;
}
__device__ __forceinline__ float ldg_f32(const float* p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

struct DeviceFixed : shade::PixelScalars {
    const float* pv;    // shared: 16 floats, column-major
    const float* pv3;   // shared: 4 floats
    const float* uvs;   // shared: 16 floats of the pixel's cascade
    const float* uvs3;  // shared: 4 floats
    const float* nt;    // global: Instance::normal_transform, 3 columns of 3
    __device__ float PV(int c, int r) const { return c == 3 ? lds_f32(pv3 + r) : lds_f32(pv + 4 * c + r); }
    __device__ float UVS(int c, int r) const { return c == 3 ? lds_f32(uvs3 + r) : lds_f32(uvs + 4 * c + r); }
    __device__ float NT(int c, int r) const { return ldg_f32(nt + 3 * c + r); }
};

// Block-shared copies of the frame's matrices for DeviceFixed.
struct FrameMats {
    float pv[16];        // combined_perspective_view
    float uvs[4][16];    // uv_space_shadow_matrices
    float rel[20];       // column 3 of PV T(cam) and of UVS_c T(cam) (rel_columns)
};

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Per-block accumulators for addresses that many pixels of a block add to
// (a material's base-colour factor, the texels of 1 x 1 constant textures):
// open addressing over 256 slots keyed by the destination address, four
// probes, then a plain global atomic.  Slots are flushed once at block end.
struct HotCache {
    unsigned long long key[kCacheSlots];
    float sum[kCacheSlots];
};

__device__ __forceinline__ void cache_add(HotCache& c, float* addr, float v) {
    const unsigned long long k = (unsigned long long)addr;
    const uint32_t h = ((uint32_t)(k >> 2) * 2654435761u) >> 24;
    for (uint32_t probe = 0; probe < 4; probe++) {
        const uint32_t s = (h + probe) & (kCacheSlots - 1u);
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(&c.key[s]);
        if (cur == 0ull) cur = atomicCAS(&c.key[s], 0ull, k);
        if (cur == 0ull || cur == k) {
            atomicAdd(&c.sum[s], v);
            return;
        }
    }
    atomicAdd(addr, v);
}

// Runs of equal keys along the warp (a warp is one row of 32 pixels, so a
// triangle or a texel covers contiguous lanes): `end` is one past the last
// lane of this lane's run, `head` marks its first lane.
#ifndef LH_RUN_SPAN
#define LH_RUN_SPAN 1
#endif
struct Run {
    uint32_t end;   // first lane after this lane's run
    uint32_t span;  // longest run of the warp (warp uniform)
    bool head;
};

__device__ __forceinline__ Run run_of(unsigned long long key) {
    const uint32_t lane = threadIdx.x;
    const unsigned long long prev = __shfl_up_sync(kFull, key, 1);
    const bool head = lane == 0 || prev != key;
    const uint32_t heads = __ballot_sync(kFull, head);
    const uint32_t later = heads & ~((2u << lane) - 1u);
    const uint32_t end = later ? (uint32_t)__ffs(later) - 1u : 32u;
    return {end, __reduce_max_sync(kFull, end - lane), head};
}

// Sums of v[i] over the lanes [lane, end) of the run: the full run sums at
// its head.  Doubling steps stop at the warp's longest run: a step of
// o >= span adds nothing for any lane (end - lane <= span), so the sums are
// those of the full five steps; the N values share each step's shuffles.
template <int N>
__device__ __forceinline__ void run_sums(float (&v)[N], const Run& r) {
    const uint32_t lane = threadIdx.x;
#if LH_RUN_SPAN
    for (uint32_t o = 1; o < r.span; o <<= 1) {
#else
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
#endif
#pragma unroll
        for (int i = 0; i < N; i++) {
            const float w = __shfl_down_sync(kFull, v[i], o);
            if (lane + o < r.end) v[i] += w;
        }
    }
}

// What the scatter needs of a differentiated pixel besides its gradients.
struct PixelOut {
    bool ok;                // differentiated (covered, no normal map)
    uint32_t packed;        // visibility ID: triangle within the view
    const Instance* inst;
    const lh_mesh_grads* rec;  // may be null
    uint32_t idx[3];
};

// Recompute the forward of pixel (x, y) from the visibility buffer and run
// the surface half of the reverse pass of shade.cuh for the upstream
// gradient at that pixel; fx, p and st carry what the geometry half needs.
// `M` holds the block's copies of the frame matrices.
__device__ __forceinline__ void pixel_backward(const FrameDev& f, const float4* grad, const lh_grad_targets& t,
                                               const FrameMats& M, uint32_t x, uint32_t y, PixelGrad<float>& g,
                                               PixelOut& o, DeviceFixed& fx, PixelParams<float>& p,
                                               shade::SurfaceState<float>& st) {
    const Uniforms& u = *f.uniforms;
    const uint32_t W = u.window_size.x, H = u.window_size.y;
    o.ok = false;
    bool active = x < W && y < H;
    unsigned long long vis = 0;
    if (active) vis = __ldcs(reinterpret_cast<const unsigned long long*>(f.visibility) + (size_t)y * W + x);
    active = active && u2f((uint32_t)(vis >> 32)) != 0.0f;
    if (!active) return;
    const float4 gp = __ldcs(grad + (size_t)y * W + x);
    const uint32_t packed = (uint32_t)vis;
    const uint32_t slot = packed & ((1u << 24) - 1u), tri = packed >> 24;
    // the slot's draw record (written by the meshlet cull): the instance and
    // the index / micro-index addresses already offset to the meshlet, so
    // the vertex loads do not wait on the reference, MeshInfo and Meshlet
    const RasterDraw rd = f.views[0].rdraws[slot];
    const Instance* inst = f.instances + rd.instance;
    const MeshInfoResolve mi = load_mesh_info_resolve(mesh_info_of(inst));
    const uint8_t* micro = reinterpret_cast<const uint8_t*>(rd.micro) + tri * 3;
    const uint32_t flags = mi.flags;
    for (int k = 0; k < 3; k++) {
        const uint32_t vi = __ldg(micro + k);
        o.idx[k] = (flags & MESH_INFO_FLAGS_32_BIT_INDICES) ? __ldg(reinterpret_cast<const uint32_t*>(rd.indices) + vi)
                                                            : __ldg(reinterpret_cast<const uint16_t*>(rd.indices) + vi);
    }
    const lh_mat4& T = inst->transform;
    for (int k = 0; k < 3; k++) {
        f3 w = world_pos(T, load_position(rd.positions, flags, o.idx[k]));
        p.W[k] = {w.x, w.y, w.z};
        f3 nr = load_normal_raw(mi.normals, flags, o.idx[k]);
        p.N[k] = {nr.x, nr.y, nr.z};
        f2 uvr = load_uv_raw(mi.uvs, flags, o.idx[k]);
        p.UV[k] = {uvr.x, uvr.y};
    }
    p.bcf = {mi.base_color_factor.x, mi.base_color_factor.y, mi.base_color_factor.z};
    p.sun = {u.sun_dir.x, u.sun_dir.y, u.sun_dir.z};
    p.light = {u.sun_intensity.x, u.sun_intensity.y, u.sun_intensity.z};
    fx.pv = M.pv;
    fx.pv3 = M.pv + 12;
    fx.nt = &inst->normal_transform.cols[0].x;
    const f2 ndc{(float)x / (float)W * 2.0f - 1.0f, (float)y / (float)H * 2.0f - 1.0f};
    fx.ndc[0] = ndc.x;
    fx.ndc[1] = ndc.y;
    fx.win[0] = (float)W;
    fx.win[1] = (float)H;
    fx.cam[0] = u.camera_pos.x;
    fx.cam[1] = u.camera_pos.y;
    fx.cam[2] = u.camera_pos.z;
    fx.ts[0] = mi.texture_scale.x;
    fx.ts[1] = mi.texture_scale.y;
    fx.toff[0] = mi.texture_offset.x;
    fx.toff[1] = mi.texture_offset.y;
    fx.thin = (flags & MESH_INFO_FLAGS_ALPHA_CLIP) ? 1u : 0u;
    fx.bias = fx.thin ? 0.000002f : 0.0f;
    fx.shadow_size = (float)f.shadow_size;
    fx.base_tex = mi.base_tex;
    fx.mr_tex = mi.mr_tex;
    fx.has_normal_map = mi.normal_tex != UNUSED_TEXTURE_INDEX;
    DeviceSampler smp{&f};
    {
        // the world position the forward interpolated, in its absolute float
        // arithmetic, picks the cascade (render_geometry.comp:183-196) and
        // places the PCF taps
        const v3<float> world = shade::forward_world(fx, p);
        uint32_t ci;
        for (ci = 0; ci < 4; ci++) {
            const lh_mat4& m = *reinterpret_cast<const lh_mat4*>(M.uvs[ci]);
            f4 sc = mul(m, f4{world.x, world.y, world.z, 1.0f});
            float ox = sc.x - 0.5f, oy = sc.y - 0.5f;
            if (fabsf(ox) < 0.5f && fabsf(oy) < 0.5f) break;
        }
        fx.cascade = ci;
        fx.uvs = M.uvs[ci > 3 ? 3 : ci];
        fx.uvs3 = fx.uvs + 12;
        // face flip, far-plane test and compare results exactly as the forward
        shade::decide_at(fx, p, world, smp);
    }
    // the continuous part in camera-relative coordinates: W - cam is
    // (nearly) exact, and PV T(cam), UVS T(cam) were formed in double
    const uint32_t layer = fx.cascade > 3 ? 3u : fx.cascade;
    fx.pv3 = M.rel;
    fx.uvs3 = M.rel + 4 + 4 * layer;
    for (int k = 0; k < 3; k++) p.W[k] = {p.W[k].x - u.camera_pos.x, p.W[k].y - u.camera_pos.y, p.W[k].z - u.camera_pos.z};
    fx.cam[0] = fx.cam[1] = fx.cam[2] = 0.0f;
    v3<float> out;
    shade::shade_surface<float>(fx, p, smp, &out, v3<float>{gp.x, gp.y, gp.z}, &g, &st);
    if (!g.differentiated) return;
    o.ok = true;
    o.packed = packed;
    o.inst = inst;
    o.rec = t.instance_grads ? reinterpret_cast<const lh_mesh_grads*>(
                                   reinterpret_cast<const uint64_t*>(t.instance_grads)[rd.instance])
                             : nullptr;
}

// The four texels of one bilinear sample (00, 10, 01, 11): run-summed along
// the warp and added to the texture's gradient image, channels [c0, c0 + nc).
// Taps that land on the same texel (1-texel-wide textures, edges) are merged
// into the first.
template <int NC>
__device__ __forceinline__ void scatter_texels(HotCache& cache, float* const base_addr[4], float v[4][NC], int c0,
                                               bool small) {
    float* a[4] = {base_addr[0], base_addr[1], base_addr[2], base_addr[3]};
#pragma unroll
    for (int q = 1; q < 4; q++)
#pragma unroll
        for (int p = 0; p < q; p++)
            if (a[q] && a[q] == a[p]) {
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    v[p][c] += v[q][c];
                    v[q][c] = 0.0f;
                }
                a[q] = nullptr;
            }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (!__any_sync(kFull, a[q] != nullptr)) continue;
        const Run r = run_of((unsigned long long)a[q]);
        float s[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) s[c] = v[q][c];
        run_sums(s, r);
        if (r.head && a[q]) {
            if (!small && ((uintptr_t)a[q] & 15u) == 0) {
                // one vector reduction per texel (the other channels add 0)
                float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                float* tc = &t.x;
#pragma unroll
                for (int c = 0; c < NC; c++) tc[c0 + c] = s[c];
                atomicAdd(reinterpret_cast<float4*>(a[q]), t);
            } else {
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    if (small) cache_add(cache, a[q] + c0 + c, s[c]);
                    else atomicAdd(a[q] + c0 + c, s[c]);
                }
            }
        }
    }
}

// Column 3 of PV T(cam) and of UVS_c T(cam) for the 4 cascades, in double
// and rounded once: rel[r] for PV, rel[4 + 4c + r] for cascade c.  Threads
// 0..19 of the block each form one entry.
__device__ __forceinline__ void rel_columns(const FrameDev& f, uint32_t tid, float* rel) {
    if (tid >= 20) return;
    const Uniforms& u = *f.uniforms;
    const lh_mat4& m = tid < 4 ? u.combined_perspective_view : f.misc->uv_space_shadow_matrices[(tid - 4) / 4];
    const uint32_t r = tid & 3u;
    const float* c0 = &m.cols[0].x;
    const float* c1 = &m.cols[1].x;
    const float* c2 = &m.cols[2].x;
    const float* c3 = &m.cols[3].x;
    const double cx = u.camera_pos.x, cy = u.camera_pos.y, cz = u.camera_pos.z;
    rel[tid] = (float)((double)c3[r] + (((double)c0[r] * cx + (double)c1[r] * cy) + (double)c2[r] * cz));
}

// One thread per pixel over 32 x kBwdRows tiles; a grid of resident blocks strides
// over the tiles.  Gradients of the three vertices of a triangle are summed
// over the triangle's run of pixels in the warp's row before the atomics;
// the light gradients stay in registers until block end; base-colour
// factors and small textures accumulate in the block's HotCache.
template <int ROWS>
__global__ void __launch_bounds__(32 * ROWS, LH_BWD_MIN_BLOCKS * 8 / ROWS)
    k_resolve_backward(FrameDev f, const float4* grad, lh_grad_targets t, uint32_t tiles_x, uint32_t n_tiles) {
    __shared__ HotCache cache;
    __shared__ float s_light[ROWS][6];
    pdl_enter();
    __shared__ __align__(16) FrameMats s_mats;
    const uint32_t tid = threadIdx.y * 32 + threadIdx.x;
    for (uint32_t s = tid; s < kCacheSlots; s += 32 * ROWS) {
        cache.key[s] = 0ull;
        cache.sum[s] = 0.0f;
    }
    if (tid < 16) s_mats.pv[tid] = (&f.uniforms->combined_perspective_view.cols[0].x)[tid];
    if (tid < 64) s_mats.uvs[tid / 16][tid % 16] = (&f.misc->uv_space_shadow_matrices[tid / 16].cols[0].x)[tid % 16];
    rel_columns(f, tid, s_mats.rel);
    __syncthreads();
    float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const uint64_t* tex_targets = reinterpret_cast<const uint64_t*>(t.texture_grads);
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t x = (tile % tiles_x) * 32 + threadIdx.x, y = (tile / tiles_x) * ROWS + threadIdx.y;
        PixelGrad<float> g;
        PixelOut o;
        DeviceFixed fx;
        PixelParams<float> p;
        shade::SurfaceState<float> st;
        pixel_backward(f, grad, t, s_mats, x, y, g, o, fx, p, st);
        if (o.ok) {
            acc[0] += g.sun.x;
            acc[1] += g.sun.y;
            acc[2] += g.sun.z;
            acc[3] += g.light.x;
            acc[4] += g.light.y;
            acc[5] += g.light.z;
        }
        const lh_mesh_grads* mg = o.ok ? o.rec : nullptr;
        // base-colour factor of the pixel's MeshInfo record
        float* bcf_dst = mg ? reinterpret_cast<float*>(mg->base_color_factor) : nullptr;
        if (__any_sync(kFull, bcf_dst != nullptr)) {
            const Run r = run_of((unsigned long long)bcf_dst);
            float b[3] = {bcf_dst ? g.bcf.x : 0.0f, bcf_dst ? g.bcf.y : 0.0f, bcf_dst ? g.bcf.z : 0.0f};
            run_sums(b, r);
            if (r.head && bcf_dst) {
                cache_add(cache, bcf_dst, b[0]);
                cache_add(cache, bcf_dst + 1, b[1]);
                cache_add(cache, bcf_dst + 2, b[2]);
            }
        }
        if (tex_targets) {
            // base colour (rgb of the texel) and metallic-roughness (g, b)
            float* ba[4] = {nullptr, nullptr, nullptr, nullptr};
            float* ma[4] = {nullptr, nullptr, nullptr, nullptr};
            bool base_small = false, mr_small = false;
            if (o.ok && g.base_index < f.n_textures && tex_targets[g.base_index]) {
                const lh_texture& tx = f.textures[g.base_index];
                float4* dst = reinterpret_cast<float4*>(tex_targets[g.base_index]);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    ba[q] = reinterpret_cast<float*>(dst + (size_t)g.base_ij[2 + (q >> 1)] * tx.width + g.base_ij[q & 1]);
                base_small = tx.width * tx.height <= kSmallTexture;
            }
            if (o.ok && g.mr_index < f.n_textures && tex_targets[g.mr_index]) {
                const lh_texture& tx = f.textures[g.mr_index];
                float4* dst = reinterpret_cast<float4*>(tex_targets[g.mr_index]);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    ma[q] = reinterpret_cast<float*>(dst + (size_t)g.mr_ij[2 + (q >> 1)] * tx.width + g.mr_ij[q & 1]);
                mr_small = tx.width * tx.height <= kSmallTexture;
            }
            scatter_texels<3>(cache, ba, g.base_texel, 0, base_small);
            scatter_texels<2>(cache, ma, g.mr_texel, 1, mr_small);  // roughness (g), metallic (b)
        }
        // the geometry half of the reverse, then the vertex attributes: one
        // run per triangle
        if (o.ok) shade::shade_geometry<float>(fx, p, st, &g);
        if (__any_sync(kFull, mg != nullptr)) {
            const Run r = run_of(mg ? (unsigned long long)o.packed : ~0ull);
            float v[24];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                v[k * 8 + 0] = g.W[k].x;
                v[k * 8 + 1] = g.W[k].y;
                v[k * 8 + 2] = g.W[k].z;
                v[k * 8 + 3] = g.N[k].x;
                v[k * 8 + 4] = g.N[k].y;
                v[k * 8 + 5] = g.N[k].z;
                v[k * 8 + 6] = g.UV[k].x;
                v[k * 8 + 7] = g.UV[k].y;
            }
            run_sums(v, r);
            if (r.head && mg) {
                const lh_mesh_grads d = *mg;
                const lh_mat4& T = o.inst->transform;
                const f3 c0{T.cols[0].x, T.cols[0].y, T.cols[0].z}, c1{T.cols[1].x, T.cols[1].y, T.cols[1].z},
                    c2{T.cols[2].x, T.cols[2].y, T.cols[2].z};
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float* vk = v + k * 8;
                    if (d.positions) {
                        // W = M3 P + t: dP = M3^T dW
                        float* p = reinterpret_cast<float*>(d.positions) + (size_t)o.idx[k] * 3;
                        const f3 gw{vk[0], vk[1], vk[2]};
                        atomicAdd(p, dot(c0, gw));
                        atomicAdd(p + 1, dot(c1, gw));
                        atomicAdd(p + 2, dot(c2, gw));
                    }
                    if (d.normals) {
                        float* p = reinterpret_cast<float*>(d.normals) + (size_t)o.idx[k] * 3;
                        atomicAdd(p, vk[3]);
                        atomicAdd(p + 1, vk[4]);
                        atomicAdd(p + 2, vk[5]);
                    }
                    if (d.uvs) {
                        float* p = reinterpret_cast<float*>(d.uvs) + (size_t)o.idx[k] * 2;
                        if (((uintptr_t)p & 7u) == 0) {
                            atomicAdd(reinterpret_cast<float2*>(p), make_float2(vk[6], vk[7]));
                        } else {
                            atomicAdd(p, vk[6]);
                            atomicAdd(p + 1, vk[7]);
                        }
                    }
                }
            }
        }
    }
    // light direction / colour: one atomic per value per block
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const float s = warp_sum(acc[i]);
        if (threadIdx.x == 0) s_light[threadIdx.y][i] = s;
    }
    __syncthreads();
    if (tid < 6) {
        float s = 0.0f;
        for (int w = 0; w < ROWS; w++) s += s_light[w][tid];
        float* dst = tid < 3 ? reinterpret_cast<float*>(t.light_dir) : reinterpret_cast<float*>(t.light_color);
        if (dst) atomicAdd(dst + (tid % 3), s);
    }
    for (uint32_t s = tid; s < kCacheSlots; s += 32 * ROWS)
        if (cache.key[s]) atomicAdd(reinterpret_cast<float*>(cache.key[s]), cache.sum[s]);
}

int g_backward_blocks_per_sm[3] = {-1, -1, -1};

template <int ROWS>
cudaError_t launch_backward_rows(const FrameDev& f, uint32_t width, uint32_t height, const float4* grad,
                                 const lh_grad_targets& t, cudaStream_t s, int& blocks_per_sm) {
    if (blocks_per_sm < 0) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_resolve_backward<ROWS>, 32 * ROWS, 0) != cudaSuccess)
            n = 1;
        blocks_per_sm = n > 0 ? n : 1;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const uint32_t tiles_x = (width + 31) / 32, tiles_y = (height + ROWS - 1) / ROWS;
    const uint32_t n_tiles = tiles_x * tiles_y;
    if (n_tiles == 0) return cudaSuccess;
    const uint32_t grid = std::min<uint32_t>(n_tiles, (uint32_t)(sms * blocks_per_sm));
    return launch_pdl(k_resolve_backward<ROWS>, dim3(grid), dim3(32, ROWS), s, f, grad, t, tiles_x, n_tiles);
}

}  // namespace

cudaError_t launch_resolve_backward(const FrameDev& f, uint32_t width, uint32_t height, const float4* grad,
                                    const lh_grad_targets& t, cudaStream_t s) {
    switch (f.backward_rows) {
        case 4: return launch_backward_rows<4>(f, width, height, grad, t, s, g_backward_blocks_per_sm[0]);
        case 16: return launch_backward_rows<16>(f, width, height, grad, t, s, g_backward_blocks_per_sm[2]);
        default: return launch_backward_rows<8>(f, width, height, grad, t, s, g_backward_blocks_per_sm[1]);
    }
}

}  // namespace lh
