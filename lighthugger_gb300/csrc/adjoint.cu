// Backward of the lighting resolve (render_geometry.comp:70-266) with the
// visibility held fixed: one thread per pixel recomputes the forward inputs
// from the visibility buffer (triangle, vertices, cascade, compare results)
// and runs the hand-written reverse pass of shade.cuh, then adds the
// gradients into the caller's buffers.  Targets every lane of a warp shares
// (light direction / colour, a material's base-colour factor) are summed
// across the warp first, so they take one atomic per warp.
#include "frame_phases.cuh"
#include "shade.cuh"

namespace lh {
namespace {

using shade::Bilinear;
using shade::PixelFixed;
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
        const uchar4* tex = reinterpret_cast<const uchar4*>(t.texels);
        float u = uv.x * (float)t.width - 0.5f, v = uv.y * (float)t.height - 0.5f;
        if (!(fabsf(u) < 1e9f)) u = 0.0f;
        if (!(fabsf(v) < 1e9f)) v = 0.0f;
        float fu = floorf(u), fv = floorf(v);
        s.a = u - fu;
        s.b = v - fv;
        long long i0 = (long long)fu, j0 = (long long)fv;
        long long W = t.width, H = t.height;
        s.i0 = ((i0 % W) + W) % W;
        s.i1 = (((i0 + 1) % W) + W) % W;
        s.j0 = ((j0 % H) + H) % H;
        s.j1 = (((j0 + 1) % H) + H) % H;
        s.size_u = (float)t.width;
        s.size_v = (float)t.height;
        auto texel = [&](long long i, long long j, float* o) {
            uchar4 p = __ldg(tex + ((size_t)j * W + i));
            if (t.srgb) { o[0] = f->srgb_lut[p.x]; o[1] = f->srgb_lut[p.y]; o[2] = f->srgb_lut[p.z]; }
            else { o[0] = (float)p.x / 255.0f; o[1] = (float)p.y / 255.0f; o[2] = (float)p.z / 255.0f; }
            o[3] = (float)p.w / 255.0f;
        };
        texel(s.i0, s.j0, s.t00);
        texel(s.i1, s.j0, s.t10);
        texel(s.i0, s.j1, s.t01);
        texel(s.i1, s.j1, s.t11);
        return s;
    }
    __device__ float shadow_cmp(uint32_t layer, int64_t i, int64_t j, float ref) const {
        const int64_t S = f->shadow_size;
        i = i < 0 ? 0 : (i > S - 1 ? S - 1 : i);
        j = j < 0 ? 0 : (j > S - 1 ? S - 1 : j);
        return ref < __ldg(f->shadow_maps + ((size_t)layer * S + j) * S + i) ? 1.0f : 0.0f;
    }
};

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Add a 3-vector to `dst` (may be null per lane): one atomic per warp when
// every lane targets the same address, else one per lane.
__device__ __forceinline__ void add3(float* dst, float x, float y, float z) {
    const unsigned long long key = (unsigned long long)dst;
    const unsigned long long k0 = __shfl_sync(0xFFFFFFFFu, key, 0);
    if (__all_sync(0xFFFFFFFFu, key == k0)) {
        x = warp_sum(x);
        y = warp_sum(y);
        z = warp_sum(z);
        if ((threadIdx.x & 31) == 0 && dst) {
            atomicAdd(dst, x);
            atomicAdd(dst + 1, y);
            atomicAdd(dst + 2, z);
        }
    } else if (dst) {
        atomicAdd(dst, x);
        atomicAdd(dst + 1, y);
        atomicAdd(dst + 2, z);
    }
}

__global__ void __launch_bounds__(256, 2) k_resolve_backward(FrameDev f, const float4* grad, lh_grad_targets t) {
    const Uniforms& u = *f.uniforms;
    const uint32_t W = u.window_size.x, H = u.window_size.y;
    const uint32_t x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    bool active = x < W && y < H;
    unsigned long long vis = 0;
    if (active) vis = __ldcs(reinterpret_cast<const unsigned long long*>(f.visibility) + (size_t)y * W + x);
    active = active && u2f((uint32_t)(vis >> 32)) != 0.0f;
    float* bcf_dst = nullptr;
    v3<float> g_sun{0.0f, 0.0f, 0.0f}, g_light{0.0f, 0.0f, 0.0f}, g_bcf{0.0f, 0.0f, 0.0f};
    if (active) {
        const float4 gp = grad[(size_t)y * W + x];
        const uint32_t packed = (uint32_t)vis;
        const uint32_t slot = packed & ((1u << 24) - 1u), tri = packed >> 24;
        const MeshletReference ref = f.views[0].refs[slot];
        const Instance* inst = f.instances + ref.instance_index;
        const MeshInfoResolve mi = load_mesh_info_resolve(mesh_info_of(inst));
        const Meshlet* ml = reinterpret_cast<const Meshlet*>(mi.meshlets) + ref.meshlet_index;
        const uint32_t tri_off = __ldg(&ml->triangle_offset), idx_off = __ldg(&ml->index_offset);
        const uint8_t* micro = reinterpret_cast<const uint8_t*>(mi.micro_indices) + tri_off + tri * 3;
        const uint32_t flags = mi.flags;
        uint32_t idx[3];
        for (int k = 0; k < 3; k++) {
            uint32_t vi = idx_off + __ldg(micro + k);
            idx[k] = (flags & MESH_INFO_FLAGS_32_BIT_INDICES) ? __ldg(reinterpret_cast<const uint32_t*>(mi.indices) + vi)
                                                              : __ldg(reinterpret_cast<const uint16_t*>(mi.indices) + vi);
        }
        const lh_mat4& T = inst->transform;
        PixelParams<float> p;
        for (int k = 0; k < 3; k++) {
            f3 w = world_pos(T, load_position(mi.positions, flags, idx[k]));
            p.W[k] = {w.x, w.y, w.z};
            f3 nr = load_normal_raw(mi.normals, flags, idx[k]);
            p.N[k] = {nr.x, nr.y, nr.z};
            f2 uvr = load_uv_raw(mi.uvs, flags, idx[k]);
            p.UV[k] = {uvr.x, uvr.y};
        }
        p.bcf = {mi.base_color_factor.x, mi.base_color_factor.y, mi.base_color_factor.z};
        p.sun = {u.sun_dir.x, u.sun_dir.y, u.sun_dir.z};
        p.light = {u.sun_intensity.x, u.sun_intensity.y, u.sun_intensity.z};
        PixelFixed fx;
        for (int c = 0; c < 4; c++) {
            fx.pv[c][0] = u.combined_perspective_view.cols[c].x;
            fx.pv[c][1] = u.combined_perspective_view.cols[c].y;
            fx.pv[c][2] = u.combined_perspective_view.cols[c].z;
            fx.pv[c][3] = u.combined_perspective_view.cols[c].w;
        }
        for (int c = 0; c < 3; c++) {
            fx.nt[c][0] = inst->normal_transform.cols[c].x;
            fx.nt[c][1] = inst->normal_transform.cols[c].y;
            fx.nt[c][2] = inst->normal_transform.cols[c].z;
        }
        // the world position the forward interpolated decides the cascade
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
        // the cascade the forward chose: its own barycentrics and world
        // position, in its absolute float arithmetic (render_geometry.comp:183-196)
        {
            f4 c0 = mul(u.combined_perspective_view, f4{p.W[0].x, p.W[0].y, p.W[0].z, 1.0f});
            f4 c1 = mul(u.combined_perspective_view, f4{p.W[1].x, p.W[1].y, p.W[1].z, 1.0f});
            f4 c2 = mul(u.combined_perspective_view, f4{p.W[2].x, p.W[2].y, p.W[2].z, 1.0f});
            f3 invW{1.0f / c0.w, 1.0f / c1.w, 1.0f / c2.w};
            f2 n0{c0.x * invW.x, c0.y * invW.x}, n1{c1.x * invW.y, c1.y * invW.y}, n2{c2.x * invW.z, c2.y * invW.z};
            f2 ca{n2.x - n1.x, n2.y - n1.y}, cb{n0.x - n1.x, n0.y - n1.y};
            float invDet = 1.0f / (ca.x * cb.y - cb.x * ca.y);
            f3 ddx = f3{n1.y - n2.y, n2.y - n0.y, n0.y - n1.y} * invDet * invW;
            f3 ddy = f3{n2.x - n1.x, n0.x - n2.x, n1.x - n0.x} * invDet * invW;
            float ddxSum = dot(ddx, f3{1.0f, 1.0f, 1.0f});
            float ddySum = dot(ddy, f3{1.0f, 1.0f, 1.0f});
            f2 dv{ndc.x - n0.x, ndc.y - n0.y};
            float interpInvW = (invW.x + dv.x * ddxSum) + dv.y * ddySum;
            float interpW = 1.0f / interpInvW;
            float l0 = interpW * ((invW.x + dv.x * ddx.x) + dv.y * ddy.x);
            float l1 = interpW * ((0.0f + dv.x * ddx.y) + dv.y * ddy.y);
            float l2 = interpW * ((0.0f + dv.x * ddx.z) + dv.y * ddy.z);
            f3 world{(p.W[0].x * l0 + p.W[1].x * l1) + p.W[2].x * l2, (p.W[0].y * l0 + p.W[1].y * l1) + p.W[2].y * l2,
                     (p.W[0].z * l0 + p.W[1].z * l1) + p.W[2].z * l2};
            uint32_t ci;
            for (ci = 0; ci < 4; ci++) {
                f4 sc = mul(f.misc->uv_space_shadow_matrices[ci], f4{world.x, world.y, world.z, 1.0f});
                float ox = sc.x - 0.5f, oy = sc.y - 0.5f;
                if (fabsf(ox) < 0.5f && fabsf(oy) < 0.5f) break;
            }
            fx.cascade = ci;
            const lh_mat4& m = f.misc->uv_space_shadow_matrices[ci > 3 ? 3 : ci];
            for (int c = 0; c < 4; c++) {
                fx.uvs[c][0] = m.cols[c].x;
                fx.uvs[c][1] = m.cols[c].y;
                fx.uvs[c][2] = m.cols[c].z;
                fx.uvs[c][3] = m.cols[c].w;
            }
        }
        DeviceSampler smp{&f};
        // face flip, far-plane test and compare results exactly as the forward
        shade::decide<float>(fx, p, smp);
        // the continuous part in camera-relative coordinates: W - cam is
        // (nearly) exact, and PV T(cam), UVS T(cam) are formed in double
        const double cx = u.camera_pos.x, cy = u.camera_pos.y, cz = u.camera_pos.z;
        for (int r = 0; r < 4; r++) {
            fx.pv[3][r] = (float)((double)fx.pv[3][r] + (((double)fx.pv[0][r] * cx + (double)fx.pv[1][r] * cy) +
                                                         (double)fx.pv[2][r] * cz));
            fx.uvs[3][r] = (float)((double)fx.uvs[3][r] + (((double)fx.uvs[0][r] * cx + (double)fx.uvs[1][r] * cy) +
                                                           (double)fx.uvs[2][r] * cz));
        }
        for (int k = 0; k < 3; k++) p.W[k] = {p.W[k].x - u.camera_pos.x, p.W[k].y - u.camera_pos.y, p.W[k].z - u.camera_pos.z};
        fx.cam[0] = fx.cam[1] = fx.cam[2] = 0.0f;
        v3<float> out;
        PixelGrad<float> g;
        shade::shade<float>(fx, p, smp, &out, v3<float>{gp.x, gp.y, gp.z}, &g);
        if (g.differentiated) {
            g_sun = g.sun;
            g_light = g.light;
            g_bcf = g.bcf;
            const uint64_t rec = t.instance_grads ? reinterpret_cast<const uint64_t*>(t.instance_grads)[ref.instance_index]
                                                  : 0ull;
            if (rec) {
                const lh_mesh_grads mg = *reinterpret_cast<const lh_mesh_grads*>(rec);
                for (int k = 0; k < 3; k++) {
                    if (mg.positions) {
                        // W = M3 P + t: dP = M3^T dW
                        float* d = reinterpret_cast<float*>(mg.positions) + (size_t)idx[k] * 3;
                        f3 gw{g.W[k].x, g.W[k].y, g.W[k].z};
                        atomicAdd(d, dot(f3{T.cols[0].x, T.cols[0].y, T.cols[0].z}, gw));
                        atomicAdd(d + 1, dot(f3{T.cols[1].x, T.cols[1].y, T.cols[1].z}, gw));
                        atomicAdd(d + 2, dot(f3{T.cols[2].x, T.cols[2].y, T.cols[2].z}, gw));
                    }
                    if (mg.normals) {
                        float* d = reinterpret_cast<float*>(mg.normals) + (size_t)idx[k] * 3;
                        atomicAdd(d, g.N[k].x);
                        atomicAdd(d + 1, g.N[k].y);
                        atomicAdd(d + 2, g.N[k].z);
                    }
                    if (mg.uvs) {
                        float* d = reinterpret_cast<float*>(mg.uvs) + (size_t)idx[k] * 2;
                        atomicAdd(d, g.UV[k].x);
                        atomicAdd(d + 1, g.UV[k].y);
                    }
                }
                bcf_dst = reinterpret_cast<float*>(mg.base_color_factor);
            }
            if (t.texture_grads) {
                // the 4 texels of each bilinear sample: 00, 10, 01, 11
                const uint64_t* tg = reinterpret_cast<const uint64_t*>(t.texture_grads);
                if (g.base_index < f.n_textures && tg[g.base_index]) {
                    const uint32_t tw = f.textures[g.base_index].width;
                    float4* dst = reinterpret_cast<float4*>(tg[g.base_index]);
                    for (int q = 0; q < 4; q++) {
                        int64_t i = g.base_ij[q & 1], j = g.base_ij[2 + (q >> 1)];
                        float* d = reinterpret_cast<float*>(dst + (size_t)j * tw + i);
                        atomicAdd(d, g.base_texel[q][0]);
                        atomicAdd(d + 1, g.base_texel[q][1]);
                        atomicAdd(d + 2, g.base_texel[q][2]);
                    }
                }
                if (g.mr_index < f.n_textures && tg[g.mr_index]) {
                    const uint32_t tw = f.textures[g.mr_index].width;
                    float4* dst = reinterpret_cast<float4*>(tg[g.mr_index]);
                    for (int q = 0; q < 4; q++) {
                        int64_t i = g.mr_ij[q & 1], j = g.mr_ij[2 + (q >> 1)];
                        float* d = reinterpret_cast<float*>(dst + (size_t)j * tw + i);
                        atomicAdd(d + 1, g.mr_texel[q][0]);  // roughness (g)
                        atomicAdd(d + 2, g.mr_texel[q][1]);  // metallic (b)
                    }
                }
            }
        }
    }
    add3(reinterpret_cast<float*>(t.light_dir), g_sun.x, g_sun.y, g_sun.z);
    add3(reinterpret_cast<float*>(t.light_color), g_light.x, g_light.y, g_light.z);
    add3(bcf_dst, g_bcf.x, g_bcf.y, g_bcf.z);
}

}  // namespace

cudaError_t launch_resolve_backward(const FrameDev& f, uint32_t width, uint32_t height, const float4* grad,
                                    const lh_grad_targets& t, cudaStream_t s) {
    dim3 grid((width + 31) / 32, (height + 7) / 8);
    k_resolve_backward<<<grid, dim3(32, 8), 0, s>>>(f, grad, t);
    return cudaGetLastError();
}

}  // namespace lh
