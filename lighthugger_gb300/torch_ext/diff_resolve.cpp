// libtorch autograd Function around the GB300 resolve and its adjoint.
//
// forward(light_dir, light_color, positions, normals, uvs, base_color_factors,
//         textures)
//   writes the parameter tensors into the scene's device buffers (the
//   buffers the MeshInfo records point at, and the context's linear copies
//   of the textures), renders one frame through the C ABI (lh_frame) with
//   Uniforms.sun_dir / sun_intensity taken from the light tensors, and
//   returns the linear HDR image [H, W, 4].
// backward(grad_hdr)
//   runs lh_resolve_backward with visibility held fixed (the forward's
//   visibility buffer, shadow maps and cascade fit) and returns the
//   gradients of the same tensors.
//
// All work is enqueued on PyTorch's current CUDA stream of the parameters'
// device (the backward on the stream autograd runs it on), so it is ordered
// with the caller's other work on that stream.  The forward waits once for
// the six light values (one device-to-host copy): the frame's Uniforms are
// host data.
//
// positions / normals / uvs are flat float32 CUDA tensors concatenating the
// vertex data of every mesh (vertex buffers shared by several MeshInfo
// records appear once); `mesh_layout` (CPU int64 [meshes, 6]) gives for mesh
// k: vertex count, first vertex in the flat tensors, device addresses of its
// position / normal / uv buffers, 1 when fp32.  bcf is [records, 3], one
// base-colour factor per MeshInfo record; `record_layout` (CPU int64
// [records, 2]) gives each record's mesh and the device address of its
// base_color_factor field; `instance_record` (CPU int64 [instances]) maps
// instances to records.  `textures` is a flat float32 CUDA tensor of every
// texture's linear RGBA texels (4 floats per texel, textures back to back in
// index order: base colour rgb, alpha; metallic-roughness g = roughness,
// b = metallic -- render_geometry.comp:233-236); `texture_layout` (CPU int64
// [textures, 2]) gives each texture's texel count and the device address of
// the context's linear copy (lh_get_texture_linear).
#include <ATen/cuda/CUDAContext.h>
#include <torch/extension.h>

#include <cuda_runtime.h>

#include <vector>

#include "lh/lh.h"

using torch::Tensor;
using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

namespace {

void check(lh_status st, lh_ctx* ctx, const char* what) {
    TORCH_CHECK(st == LH_OK, what, " failed with status ", st, ": ", lh_last_error(ctx));
}

void check_cuda(cudaError_t e, const char* what) { TORCH_CHECK(e == cudaSuccess, what, ": ", cudaGetErrorString(e)); }

struct MeshLayout {
    int64_t vertices, first, pos, nrm, uv, fp32;
};

std::vector<MeshLayout> read_meshes(const Tensor& layout) {
    TORCH_CHECK(layout.device().is_cpu() && layout.scalar_type() == torch::kInt64 && layout.dim() == 2 &&
                    layout.size(1) == 6,
                "mesh_layout must be a CPU int64 [meshes, 6] tensor");
    auto a = layout.accessor<int64_t, 2>();
    std::vector<MeshLayout> out;
    for (int64_t k = 0; k < layout.size(0); k++) out.push_back({a[k][0], a[k][1], a[k][2], a[k][3], a[k][4], a[k][5]});
    return out;
}

void check_texture_layout(const Tensor& layout, const Tensor& textures) {
    TORCH_CHECK(layout.device().is_cpu() && layout.scalar_type() == torch::kInt64 && layout.dim() == 2 &&
                    layout.size(1) == 2,
                "texture_layout must be a CPU int64 [textures, 2] tensor");
    auto a = layout.accessor<int64_t, 2>();
    int64_t texels = 0;
    for (int64_t i = 0; i < layout.size(0); i++) texels += a[i][0];
    TORCH_CHECK(textures.numel() == 4 * texels, "textures must hold 4 floats per texel of texture_layout");
}

cudaStream_t current_stream(const Tensor& t) { return at::cuda::getCurrentCUDAStream(t.device().index()).stream(); }

class ResolveFunction : public torch::autograd::Function<ResolveFunction> {
   public:
    static Tensor forward(AutogradContext* actx, int64_t ctx_handle, Tensor uniforms, Tensor mesh_layout,
                          Tensor record_layout, Tensor instance_record, Tensor texture_layout, Tensor light_dir,
                          Tensor light_color, Tensor positions, Tensor normals, Tensor uvs, Tensor bcf,
                          Tensor textures) {
        lh_ctx* ctx = reinterpret_cast<lh_ctx*>(ctx_handle);
        TORCH_CHECK(uniforms.device().is_cpu() && uniforms.scalar_type() == torch::kUInt8 &&
                        uniforms.numel() == (int64_t)sizeof(Uniforms),
                    "uniforms must be a CPU uint8 tensor of sizeof(Uniforms)");
        for (const Tensor* t : {&light_dir, &light_color, &positions, &normals, &uvs, &bcf, &textures})
            TORCH_CHECK(t->is_cuda() && t->scalar_type() == torch::kFloat32 && t->is_contiguous() &&
                            t->device() == positions.device(),
                        "parameters must be contiguous float32 tensors on one CUDA device");
        TORCH_CHECK(light_dir.numel() == 3 && light_color.numel() == 3, "light_dir and light_color hold 3 floats");
        TORCH_CHECK(record_layout.device().is_cpu() && record_layout.scalar_type() == torch::kInt64 &&
                        record_layout.dim() == 2 && record_layout.size(1) == 2 && bcf.size(0) == record_layout.size(0),
                    "record_layout must be a CPU int64 [records, 2] tensor matching bcf");
        check_texture_layout(texture_layout, textures);
        const auto meshes = read_meshes(mesh_layout);
        cudaStream_t stream = current_stream(positions);
        // parameters -> scene buffers
        for (size_t k = 0; k < meshes.size(); k++) {
            const MeshLayout& m = meshes[k];
            TORCH_CHECK(m.fp32 == 1, "mesh ", k, " has quantized attributes; differentiate fp32 meshes");
            TORCH_CHECK((m.first + m.vertices) * 3 <= positions.numel(), "mesh_layout exceeds positions");
            const float* p = positions.data_ptr<float>() + m.first * 3;
            const float* n = normals.data_ptr<float>() + m.first * 3;
            const float* u = uvs.data_ptr<float>() + m.first * 2;
            check_cuda(cudaMemcpyAsync((void*)m.pos, p, m.vertices * 12, cudaMemcpyDeviceToDevice, stream), "copy");
            check_cuda(cudaMemcpyAsync((void*)m.nrm, n, m.vertices * 12, cudaMemcpyDeviceToDevice, stream), "copy");
            check_cuda(cudaMemcpyAsync((void*)m.uv, u, m.vertices * 8, cudaMemcpyDeviceToDevice, stream), "copy");
        }
        auto rl = record_layout.accessor<int64_t, 2>();
        for (int64_t r = 0; r < record_layout.size(0); r++)
            check_cuda(cudaMemcpyAsync((void*)rl[r][1], bcf.data_ptr<float>() + 3 * r, 12, cudaMemcpyDeviceToDevice,
                                       stream),
                       "copy");
        auto tl = texture_layout.accessor<int64_t, 2>();
        int64_t first = 0;
        for (int64_t i = 0; i < texture_layout.size(0); i++) {
            check_cuda(cudaMemcpyAsync((void*)tl[i][1], textures.data_ptr<float>() + 4 * first, 16 * tl[i][0],
                                       cudaMemcpyDeviceToDevice, stream),
                       "copy texture");
            first += tl[i][0];
        }
        Uniforms u;
        std::memcpy(&u, uniforms.data_ptr<uint8_t>(), sizeof(Uniforms));
        // the light enters the frame's host Uniforms: one copy of the six
        // values, ordered on the current stream
        Tensor light = torch::cat({light_dir.detach(), light_color.detach()}).to(torch::kCPU);
        const float* l = light.data_ptr<float>();
        u.sun_dir = {l[0], l[1], l[2]};
        u.sun_intensity = {l[3], l[4], l[5]};
        lh_frame_out out;
        check(lh_frame(ctx, &u, stream, &out), ctx, "lh_frame");
        Tensor hdr = torch::empty({(int64_t)out.height, (int64_t)out.width, 4},
                                  torch::TensorOptions().dtype(torch::kFloat32).device(positions.device()));
        check_cuda(cudaMemcpyAsync(hdr.data_ptr<float>(), (const void*)out.hdr, hdr.numel() * 4,
                                   cudaMemcpyDeviceToDevice, stream),
                   "copy hdr");
        actx->saved_data["ctx"] = ctx_handle;
        actx->save_for_backward({mesh_layout, record_layout, instance_record, texture_layout, positions, normals, uvs,
                                 bcf, light_dir, textures});
        return hdr;
    }

    static variable_list backward(AutogradContext* actx, variable_list grads) {
        lh_ctx* ctx = reinterpret_cast<lh_ctx*>(actx->saved_data["ctx"].toInt());
        auto saved = actx->get_saved_variables();
        const Tensor &mesh_layout = saved[0], &record_layout = saved[1], &instance_record = saved[2],
                     &texture_layout = saved[3], &positions = saved[4], &normals = saved[5], &uvs = saved[6],
                     &bcf = saved[7], &light_dir = saved[8], &textures = saved[9];
        const auto meshes = read_meshes(mesh_layout);
        cudaStream_t stream = current_stream(positions);
        Tensor g_hdr = grads[0].contiguous().to(torch::kFloat32);
        Tensor g_pos = torch::zeros_like(positions), g_nrm = torch::zeros_like(normals), g_uv = torch::zeros_like(uvs);
        Tensor g_tex = torch::zeros_like(textures);
        const int64_t n_rec = record_layout.size(0);
        Tensor g_bcf = torch::zeros({n_rec, 4}, bcf.options());
        Tensor g_light = torch::zeros({8}, light_dir.options());
        // one lh_mesh_grads record per MeshInfo record, one record address per instance
        Tensor records = torch::empty({n_rec, 4}, torch::kInt64);
        auto r = records.accessor<int64_t, 2>();
        auto rl = record_layout.accessor<int64_t, 2>();
        for (int64_t k = 0; k < n_rec; k++) {
            const MeshLayout& m = meshes.at((size_t)rl[k][0]);
            r[k][0] = (int64_t)(g_pos.data_ptr<float>() + m.first * 3);
            r[k][1] = (int64_t)(g_nrm.data_ptr<float>() + m.first * 3);
            r[k][2] = (int64_t)(g_uv.data_ptr<float>() + m.first * 2);
            r[k][3] = (int64_t)(g_bcf.data_ptr<float>() + 4 * k);
        }
        Tensor records_dev = records.to(positions.device());
        Tensor inst = instance_record.to(torch::kInt64).cpu().contiguous();
        Tensor inst_rec = torch::empty({inst.numel()}, torch::kInt64);
        auto ia = inst.accessor<int64_t, 1>();
        auto ra = inst_rec.accessor<int64_t, 1>();
        for (int64_t i = 0; i < inst.numel(); i++)
            ra[i] = (ia[i] < 0 || ia[i] >= n_rec) ? 0 : (int64_t)(records_dev.data_ptr<int64_t>() + 4 * ia[i]);
        Tensor inst_rec_dev = inst_rec.to(positions.device());
        // one gradient image per texture, slices of g_tex in index order
        const int64_t n_tex = texture_layout.size(0);
        Tensor tex_tab = torch::empty({std::max<int64_t>(1, n_tex)}, torch::kInt64);
        auto tl = texture_layout.accessor<int64_t, 2>();
        auto ta = tex_tab.accessor<int64_t, 1>();
        int64_t first = 0;
        for (int64_t i = 0; i < n_tex; i++) {
            ta[i] = (int64_t)(g_tex.data_ptr<float>() + 4 * first);
            first += tl[i][0];
        }
        Tensor tex_tab_dev = tex_tab.to(positions.device());
        lh_grad_targets t;
        t.instance_grads = (uint64_t)inst_rec_dev.data_ptr<int64_t>();
        t.texture_grads = n_tex ? (uint64_t)tex_tab_dev.data_ptr<int64_t>() : 0;
        t.light_dir = (uint64_t)g_light.data_ptr<float>();
        t.light_color = (uint64_t)(g_light.data_ptr<float>() + 4);
        check(lh_resolve_backward(ctx, (uint64_t)g_hdr.data_ptr<float>(), &t, stream), ctx, "lh_resolve_backward");
        return {Tensor(), Tensor(), Tensor(), Tensor(), Tensor(), Tensor(), g_light.narrow(0, 0, 3).contiguous(),
                g_light.narrow(0, 4, 3).contiguous(), g_pos, g_nrm, g_uv, g_bcf.narrow(1, 0, 3).contiguous(), g_tex};
    }
};

Tensor resolve(int64_t ctx_handle, Tensor uniforms, Tensor mesh_layout, Tensor record_layout, Tensor instance_record,
               Tensor texture_layout, Tensor light_dir, Tensor light_color, Tensor positions, Tensor normals,
               Tensor uvs, Tensor bcf, Tensor textures) {
    return ResolveFunction::apply(ctx_handle, uniforms, mesh_layout, record_layout, instance_record, texture_layout,
                                  light_dir, light_color, positions, normals, uvs, bcf, textures);
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("resolve", &resolve, "Differentiable GB300 lighting resolve (visibility held fixed)");
}
