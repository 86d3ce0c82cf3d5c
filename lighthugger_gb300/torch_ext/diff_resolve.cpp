// libtorch autograd Function around the GB300 resolve and its adjoint.
//
// forward(light_dir, light_color, positions, normals, uvs, base_color_factors)
//   writes the parameter tensors into the scene's device buffers (the
//   buffers the MeshInfo records point at), renders one frame through the C
//   ABI (lh_frame) with Uniforms.sun_dir / sun_intensity taken from the light
//   tensors, and returns the linear HDR image [H, W, 4].
// backward(grad_hdr)
//   runs lh_resolve_backward with visibility held fixed (the forward's
//   visibility buffer, shadow maps and cascade fit) and returns the
//   gradients of the same tensors.
//
// positions / normals / uvs are flat float32 CUDA tensors concatenating the
// vertex data of every mesh (vertex buffers shared by several MeshInfo
// records appear once); `mesh_layout` (CPU int64 [meshes, 6]) gives for mesh
// k: vertex count, first vertex in the flat tensors, device addresses of its
// position / normal / uv buffers, 1 when fp32.  bcf is [records, 3], one
// base-colour factor per MeshInfo record; `record_layout` (CPU int64
// [records, 2]) gives each record's mesh and the device address of its
// base_color_factor field; `instance_record` (CPU int64 [instances]) maps
// instances to records.
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

class ResolveFunction : public torch::autograd::Function<ResolveFunction> {
   public:
    static Tensor forward(AutogradContext* actx, int64_t ctx_handle, Tensor uniforms, Tensor mesh_layout,
                          Tensor record_layout, Tensor instance_record, Tensor light_dir, Tensor light_color,
                          Tensor positions, Tensor normals, Tensor uvs, Tensor bcf) {
        lh_ctx* ctx = reinterpret_cast<lh_ctx*>(ctx_handle);
        TORCH_CHECK(uniforms.device().is_cpu() && uniforms.scalar_type() == torch::kUInt8 &&
                        uniforms.numel() == (int64_t)sizeof(Uniforms),
                    "uniforms must be a CPU uint8 tensor of sizeof(Uniforms)");
        for (const Tensor* t : {&light_dir, &light_color, &positions, &normals, &uvs, &bcf})
            TORCH_CHECK(t->is_cuda() && t->scalar_type() == torch::kFloat32 && t->is_contiguous(),
                        "parameters must be contiguous float32 CUDA tensors");
        TORCH_CHECK(record_layout.device().is_cpu() && record_layout.scalar_type() == torch::kInt64 &&
                        record_layout.dim() == 2 && record_layout.size(1) == 2 && bcf.size(0) == record_layout.size(0),
                    "record_layout must be a CPU int64 [records, 2] tensor matching bcf");
        const auto meshes = read_meshes(mesh_layout);
        cudaStream_t stream = nullptr;  // legacy default stream, the one torch's default work runs on
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
        Uniforms u;
        std::memcpy(&u, uniforms.data_ptr<uint8_t>(), sizeof(Uniforms));
        Tensor ld = light_dir.detach().cpu(), lc = light_color.detach().cpu();
        u.sun_dir = {ld[0].item<float>(), ld[1].item<float>(), ld[2].item<float>()};
        u.sun_intensity = {lc[0].item<float>(), lc[1].item<float>(), lc[2].item<float>()};
        lh_frame_out out;
        check(lh_frame(ctx, &u, stream, &out), ctx, "lh_frame");
        Tensor hdr = torch::empty({(int64_t)out.height, (int64_t)out.width, 4},
                                  torch::TensorOptions().dtype(torch::kFloat32).device(positions.device()));
        check_cuda(cudaMemcpyAsync(hdr.data_ptr<float>(), (const void*)out.hdr, hdr.numel() * 4,
                                   cudaMemcpyDeviceToDevice, stream),
                   "copy hdr");
        actx->saved_data["ctx"] = ctx_handle;
        actx->save_for_backward({mesh_layout, record_layout, instance_record, positions, normals, uvs, bcf, light_dir});
        return hdr;
    }

    static variable_list backward(AutogradContext* actx, variable_list grads) {
        lh_ctx* ctx = reinterpret_cast<lh_ctx*>(actx->saved_data["ctx"].toInt());
        auto saved = actx->get_saved_variables();
        const Tensor &mesh_layout = saved[0], &record_layout = saved[1], &instance_record = saved[2],
                     &positions = saved[3], &normals = saved[4], &uvs = saved[5], &bcf = saved[6],
                     &light_dir = saved[7];
        const auto meshes = read_meshes(mesh_layout);
        Tensor g_hdr = grads[0].contiguous().to(torch::kFloat32);
        Tensor g_pos = torch::zeros_like(positions), g_nrm = torch::zeros_like(normals), g_uv = torch::zeros_like(uvs);
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
        lh_grad_targets t;
        t.instance_grads = (uint64_t)inst_rec_dev.data_ptr<int64_t>();
        t.texture_grads = 0;
        t.light_dir = (uint64_t)g_light.data_ptr<float>();
        t.light_color = (uint64_t)(g_light.data_ptr<float>() + 4);
        check(lh_resolve_backward(ctx, (uint64_t)g_hdr.data_ptr<float>(), &t, nullptr), ctx, "lh_resolve_backward");
        return {Tensor(), Tensor(), Tensor(), Tensor(), Tensor(), g_light.narrow(0, 0, 3).contiguous(),
                g_light.narrow(0, 4, 3).contiguous(), g_pos, g_nrm, g_uv, g_bcf.narrow(1, 0, 3).contiguous()};
    }
};

Tensor resolve(int64_t ctx_handle, Tensor uniforms, Tensor mesh_layout, Tensor record_layout, Tensor instance_record,
               Tensor light_dir, Tensor light_color, Tensor positions, Tensor normals, Tensor uvs, Tensor bcf) {
    return ResolveFunction::apply(ctx_handle, uniforms, mesh_layout, record_layout, instance_record, light_dir,
                                  light_color, positions, normals, uvs, bcf);
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("resolve", &resolve, "Differentiable GB300 lighting resolve (visibility held fixed)");
}
