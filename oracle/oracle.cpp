// CPU oracle of the visibility pipeline -- TEST INFRASTRUCTURE ONLY.
// Restates the reference's GLSL passes one by one; each function cites the
// reference file:line it follows (paths inside expenses/lighthugger).  Built
// with -ffp-contract=off so every float operation rounds on its own.
// Parity against the reference itself is UNPINNED (see oracle.h).
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------ GLSL-like types
template <class T> struct V2 { T x, y; };
template <class T> struct V3 { T x, y, z; };
template <class T> struct V4 { T x, y, z, w; };
template <class T> static V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> static V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> static V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> static V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> static V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> static V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> static T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> static T sqrt_(T x) { return std::sqrt(x); }
template <class T> static T length(V3<T> v) { return sqrt_(dot(v, v)); }
template <class T> static V3<T> normalize(V3<T> v) { T l = length(v); return {v.x / l, v.y / l, v.z / l}; }
template <class T> static V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> static T clampf(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }

using vec2 = V2<float>;
using vec3 = V3<float>;
using vec4 = V4<float>;

template <class T> static V3<T> v3(const lh_vec3& a) { return {(T)a.x, (T)a.y, (T)a.z}; }
template <class T> static V4<T> col(const lh_mat4& m, int c) {
    return {(T)m.cols[c].x, (T)m.cols[c].y, (T)m.cols[c].z, (T)m.cols[c].w};
}
// mat4 * vec4, ((c0*x + c1*y) + c2*z) + c3*w per row.
template <class T> static V4<T> mul(const lh_mat4& m, V4<T> v) {
    V4<T> c0 = col<T>(m, 0), c1 = col<T>(m, 1), c2 = col<T>(m, 2), c3 = col<T>(m, 3);
    return {((c0.x * v.x + c1.x * v.y) + c2.x * v.z) + c3.x * v.w,
            ((c0.y * v.x + c1.y * v.y) + c2.y * v.z) + c3.y * v.w,
            ((c0.z * v.x + c1.z * v.y) + c2.z * v.z) + c3.z * v.w,
            ((c0.w * v.x + c1.w * v.y) + c2.w * v.z) + c3.w * v.w};
}
template <class T> static V3<T> mul3(const lh_mat3& m, V3<T> v) {
    V3<T> c0 = v3<T>(m.cols[0]), c1 = v3<T>(m.cols[1]), c2 = v3<T>(m.cols[2]);
    return {(c0.x * v.x + c1.x * v.y) + c2.x * v.z, (c0.y * v.x + c1.y * v.y) + c2.y * v.z,
            (c0.z * v.x + c1.z * v.y) + c2.z * v.z};
}
static lh_mat4 matmul(const lh_mat4& a, const lh_mat4& b) {
    lh_mat4 r;
    for (int c = 0; c < 4; c++) {
        vec4 v = mul<float>(a, col<float>(b, c));
        r.cols[c] = {v.x, v.y, v.z, v.w};
    }
    return r;
}

static float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// ------------------------------------------------------------ threading
struct Pool {
    int n;
    explicit Pool(int threads) : n(threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency())) {}
    // Run f(begin, end) over [0, count) in chunks; deterministic results are
    // the caller's business (only order-independent reductions / disjoint writes).
    void run(size_t count, size_t chunk, const std::function<void(size_t, size_t)>& f) {
        if (count == 0) return;
        std::atomic<size_t> next{0};
        auto worker = [&]() {
            for (;;) {
                size_t b = next.fetch_add(chunk);
                if (b >= count) break;
                f(b, std::min(count, b + chunk));
            }
        };
        int nt = (int)std::min<size_t>((size_t)n, (count + chunk - 1) / chunk);
        std::vector<std::thread> ts;
        for (int i = 1; i < nt; i++) ts.emplace_back(worker);
        worker();
        for (auto& t : ts) t.join();
    }
};

static void atomic_max_u64(uint64_t* p, uint64_t v) {
    auto* a = reinterpret_cast<std::atomic<uint64_t>*>(p);
    uint64_t cur = a->load(std::memory_order_relaxed);
    while (v > cur && !a->compare_exchange_weak(cur, v, std::memory_order_relaxed)) {}
}
static void atomic_min_u32(uint32_t* p, uint32_t v) {
    auto* a = reinterpret_cast<std::atomic<uint32_t>*>(p);
    uint32_t cur = a->load(std::memory_order_relaxed);
    while (v < cur && !a->compare_exchange_weak(cur, v, std::memory_order_relaxed)) {}
}

// ------------------------------------------------------------ scene access (BDA views)
static const MeshInfo& mesh_info_of(const Instance& inst) {
    return *reinterpret_cast<const MeshInfo*>((uintptr_t)inst.mesh_info_address);
}
static const Meshlet& meshlet_of(const MeshInfo& mi, uint32_t i) {
    return reinterpret_cast<const Meshlet*>((uintptr_t)mi.meshlets)[i];
}
// util.glsl:3-9
static uint32_t load_index(const MeshInfo& mi, uint32_t vertex_id) {
    if (mi.flags & MESH_INFO_FLAGS_32_BIT_INDICES) return reinterpret_cast<const uint32_t*>((uintptr_t)mi.indices)[vertex_id];
    return reinterpret_cast<const uint16_t*>((uintptr_t)mi.indices)[vertex_id];
}
// QuantizedPositionBuffer (buffer_references.glsl:29-32), or f32x3 with the FP32 flag.
template <class T> static V3<T> load_position(const MeshInfo& mi, uint32_t index) {
    if (mi.flags & MESH_INFO_FLAGS_FP32_VERTICES) {
        const float* p = reinterpret_cast<const float*>((uintptr_t)mi.positions) + (size_t)index * 3;
        return {(T)p[0], (T)p[1], (T)p[2]};
    }
    const uint16_t* p = reinterpret_cast<const uint16_t*>((uintptr_t)mi.positions) + (size_t)index * 3;
    return {(T)(float)p[0], (T)(float)p[1], (T)(float)p[2]};
}
template <class T> static V3<T> load_normal_raw(const MeshInfo& mi, uint32_t index) {
    if (mi.flags & MESH_INFO_FLAGS_FP32_VERTICES) {
        const float* p = reinterpret_cast<const float*>((uintptr_t)mi.normals) + (size_t)index * 3;
        return {(T)p[0], (T)p[1], (T)p[2]};
    }
    const int8_t* p = reinterpret_cast<const int8_t*>((uintptr_t)mi.normals) + (size_t)index * 3;
    return {(T)(float)p[0], (T)(float)p[1], (T)(float)p[2]};
}
template <class T> static V2<T> load_uv_raw(const MeshInfo& mi, uint32_t index) {
    if (mi.flags & MESH_INFO_FLAGS_FP32_VERTICES) {
        const float* p = reinterpret_cast<const float*>((uintptr_t)mi.uvs) + (size_t)index * 2;
        return {(T)p[0], (T)p[1]};
    }
    const uint16_t* p = reinterpret_cast<const uint16_t*>((uintptr_t)mi.uvs) + (size_t)index * 2;
    return {(T)(float)p[0], (T)(float)p[1]};
}
// util.glsl:11-16
template <class T> static V3<T> calculate_world_pos(const Instance& inst, const MeshInfo& mi, uint32_t index) {
    V3<T> p = load_position<T>(mi, index);
    V4<T> w = mul<T>(inst.transform, V4<T>{p.x, p.y, p.z, (T)1});
    return {w.x, w.y, w.z};
}

// ------------------------------------------------------------ culling.glsl
// culling.glsl:1-46
static bool cull_bounding_sphere(const Uniforms& u, const Instance& inst, lh_vec4 bs) {
    vec4 w4 = mul<float>(inst.transform, vec4{bs.x, bs.y, bs.z, 1.0f});
    vec3 world{w4.x, w4.y, w4.z};
    float radius = bs.w;
    vec3 scale{length(v3<float>({inst.transform.cols[0].x, inst.transform.cols[0].y, inst.transform.cols[0].z})),
               length(v3<float>({inst.transform.cols[1].x, inst.transform.cols[1].y, inst.transform.cols[1].z})),
               length(v3<float>({inst.transform.cols[2].x, inst.transform.cols[2].y, inst.transform.cols[2].z}))};
    float scale_scalar = std::max(std::max(scale.x, scale.y), scale.z);
    radius *= scale_scalar;
    vec4 vs = mul<float>(u.initial_view, vec4{world.x, world.y, world.z, 1.0f});
    vs.z = -vs.z;
    bool visible = vs.z + radius > NEAR_PLANE;
    // transpose(perspective)[3].xyz + transpose(perspective)[k].xyz = row 3 + row k
    const lh_mat4& P = u.perspective;
    vec3 fx = normalize(vec3{P.cols[0].w + P.cols[0].x, P.cols[1].w + P.cols[1].x, P.cols[2].w + P.cols[2].x});
    vec3 fy = normalize(vec3{P.cols[0].w + P.cols[0].y, P.cols[1].w + P.cols[1].y, P.cols[2].w + P.cols[2].y});
    visible = visible && vs.z * fx.z + std::fabs(vs.x) * fx.x < radius;
    visible = visible && vs.z * fy.z - std::fabs(vs.y) * fy.y < radius;
    return !visible;
}
// culling.glsl:48-62
static bool fits_partially_inside(vec2 p, float r, float size) {
    return (std::fabs(p.x) - r < size) && (std::fabs(p.y) - r < size);
}
static bool fits_entirely_inside(vec2 p, float r, float size) {
    return (std::fabs(p.x) + r < size) && (std::fabs(p.y) + r < size);
}
// culling.glsl:64-80
static bool fits_entirely_inside_cascade(const MiscStorage& m, vec3 world, float r, uint32_t c) {
    vec4 v = mul<float>(m.shadow_view_matrices[c], vec4{world.x, world.y, world.z, 1.0f});
    return fits_entirely_inside(vec2{v.x, v.y}, r, m.shadow_sphere_radii[c]);
}
// culling.glsl:82-135
static bool cull_bounding_sphere_shadows(const MiscStorage& m, const Instance& inst, lh_vec4 bs, uint32_t c) {
    vec4 w4 = mul<float>(inst.transform, vec4{bs.x, bs.y, bs.z, 1.0f});
    vec3 world{w4.x, w4.y, w4.z};
    float radius = bs.w;
    vec3 scale{length(v3<float>({inst.transform.cols[0].x, inst.transform.cols[0].y, inst.transform.cols[0].z})),
               length(v3<float>({inst.transform.cols[1].x, inst.transform.cols[1].y, inst.transform.cols[1].z})),
               length(v3<float>({inst.transform.cols[2].x, inst.transform.cols[2].y, inst.transform.cols[2].z}))};
    radius *= std::max(std::max(scale.x, scale.y), scale.z);
    vec4 v = mul<float>(m.shadow_view_matrices[c], vec4{world.x, world.y, world.z, 1.0f});
    if (!fits_partially_inside(vec2{v.x, v.y}, radius, m.shadow_sphere_radii[c])) return true;
    if (c > 0 && fits_entirely_inside_cascade(m, world, radius, 0)) return true;
    if (c > 1 && fits_entirely_inside_cascade(m, world, radius, 1)) return true;
    if (c > 2 && fits_entirely_inside_cascade(m, world, radius, 2)) return true;
    return false;
}
// culling.glsl:137-145
static bool cull_cone_perspective(const Uniforms& u, const Instance& inst, const Meshlet& ml) {
    vec4 a4 = mul<float>(inst.transform, vec4{ml.cone_apex.x, ml.cone_apex.y, ml.cone_apex.z, 1.0f});
    vec3 apex{a4.x, a4.y, a4.z};
    vec3 axis = normalize(mul3<float>(inst.normal_transform, v3<float>(ml.cone_axis)));
    return dot(normalize(apex - v3<float>(u.camera_pos)), normalize(axis)) >= ml.cone_cutoff;
}
// culling.glsl:147-151
static bool cull_cone_orthographic(const Uniforms& u, const Instance& inst, const Meshlet& ml) {
    vec3 axis = normalize(mul3<float>(inst.normal_transform, v3<float>(ml.cone_axis)));
    return dot(v3<float>(u.sun_dir), axis) >= ml.cone_cutoff;
}

// ------------------------------------------------------------ prefix_sum.glsl
struct Sector {
    uint8_t* base;
    uint64_t& counter() { return *reinterpret_cast<uint64_t*>(base); }
    PrefixSumValue* values() { return reinterpret_cast<PrefixSumValue*>(base + 8); }
};
// prefix_sum.glsl:17-30, in canonical (ascending instance) order.
static void prefix_sum_inclusive_append(Sector s, uint32_t capacity, uint32_t index, uint32_t value, uint32_t* flags) {
    uint64_t old = s.counter();
    s.counter() = old + ((uint64_t)value | (1ull << 32));
    uint32_t bi = (uint32_t)(old >> 32);
    if (bi >= capacity) { *flags |= LH_FLAG_INSTANCE_OVERFLOW; return; }
    s.values()[bi].index = index;
    s.values()[bi].sum = (uint32_t)old + value;
}
// prefix_sum.glsl:33-46 (upper_bound over inclusive sums)
static PrefixSumValue prefix_sum_binary_search(Sector s, uint32_t capacity, uint32_t target) {
    uint32_t count = std::min((uint32_t)(s.counter() >> 32), capacity);
    uint32_t first = 0;
    while (count > 0) {
        uint32_t step = count / 2;
        uint32_t current = first + step;
        bool greater = target >= s.values()[current].sum;
        first = greater ? current + 1 : first;
        count = greater ? count - (step + 1) : step;
    }
    return s.values()[first];
}

// ------------------------------------------------------------ meshlet cull (write_draw_calls.comp)
struct ViewLists {
    MeshletReference* refs;  // 2*max_draws
    uint8_t* draw_section;   // {u32 num_opaque, u32 num_alpha, DrawIndirectCommand[2*max_draws]}
    uint32_t& num_opaque() { return *reinterpret_cast<uint32_t*>(draw_section); }
    uint32_t& num_alpha() { return *reinterpret_cast<uint32_t*>(draw_section + 4); }
    DrawIndirectCommand* draws() { return reinterpret_cast<DrawIndirectCommand*>(draw_section + 8); }
};

struct Frame {
    const lho_frame_desc* d;
    lho_frame_out* o;
    Pool pool;
    uint32_t W, H, S;
    size_t sector_bytes, draw_bytes;
    explicit Frame(const lho_frame_desc* d_, lho_frame_out* o_) : d(d_), o(o_), pool(d_->threads) {
        W = d->uniforms->window_size.x;
        H = d->uniforms->window_size.y;
        S = d->shadow_size;
        sector_bytes = 8 + 8 * (size_t)d->max_instances;
        draw_bytes = 8 + 16 * 2 * (size_t)d->max_draws;
    }
    Sector sector(uint32_t v) { return Sector{o->prefix_sums + v * sector_bytes}; }
    ViewLists lists(uint32_t v) {
        return ViewLists{o->meshlet_references + (size_t)v * 2 * d->max_draws, o->draw_calls + v * draw_bytes};
    }
};

// write_draw_calls.comp:7-57 (view 0) and :61-117 (cascade c = view-1).
// The reference appends with atomicAdd (race order); the oracle appends in
// ascending candidate-id order, the canonical order the kernels reproduce.
static void write_draw_calls(Frame& F, uint32_t view) {
    const Uniforms& u = *F.d->uniforms;
    Sector s = F.sector(view);
    uint32_t total = (uint32_t)s.counter();
    uint32_t cap = F.d->max_instances;
    // An overflowing sector holds only its first `cap` entries; candidates
    // stop at the last stored inclusive sum.
    if ((uint32_t)(s.counter() >> 32) > cap) total = cap ? s.values()[cap - 1].sum : 0;
    std::vector<uint8_t> cls(total);  // 0 culled, 1 opaque, 2 alpha clip
    std::vector<MeshletReference> refs(total);
    F.pool.run(total, 4096, [&](size_t b, size_t e) {
        for (size_t id = b; id < e; id++) {
            // util.glsl:42-59
            PrefixSumValue r = prefix_sum_binary_search(s, cap, (uint32_t)id);
            const Instance& inst = F.d->instances[r.index];
            const MeshInfo& mi = mesh_info_of(inst);
            uint32_t local = (uint32_t)id - (r.sum - mi.num_meshlets);
            MeshletReference ref;
            ref.instance_index = r.index;
            ref.meshlet_index = (uint16_t)local;
            refs[id] = ref;
            const Meshlet& ml = meshlet_of(mi, ref.meshlet_index);
            bool alpha = (mi.flags & MESH_INFO_FLAGS_ALPHA_CLIP) != 0;
            uint8_t c = 0;
            if (view == 0) {
                if (!cull_bounding_sphere(u, inst, ml.bounding_sphere) && (alpha || !cull_cone_perspective(u, inst, ml)))
                    c = alpha ? 2 : 1;
            } else {
                uint32_t cascade = view - 1;
                if (!cull_bounding_sphere_shadows(*F.o->misc, inst, ml.bounding_sphere, cascade) &&
                    (alpha || !cull_cone_orthographic(u, inst, ml)))
                    c = alpha ? 2 : 1;
            }
            cls[id] = c;
        }
    });
    ViewLists L = F.lists(view);
    uint32_t md = F.d->max_draws;
    uint32_t section_base = view * 2 * md;
    for (uint32_t id = 0; id < total; id++) {
        if (!cls[id]) continue;
        const Meshlet& ml = meshlet_of(mesh_info_of(F.d->instances[refs[id].instance_index]), refs[id].meshlet_index);
        uint32_t slot;
        if (cls[id] == 2) {
            uint32_t n = L.num_alpha()++;
            if (n >= md) { F.o->flags |= LH_FLAG_DRAW_OVERFLOW; continue; }
            slot = md + n;  // ALPHA_CLIP_DRAWS_OFFSET
        } else {
            uint32_t n = L.num_opaque()++;
            if (n >= md) { F.o->flags |= LH_FLAG_DRAW_OVERFLOW; continue; }
            slot = n;
        }
        DrawIndirectCommand dc;
        dc.vertexCount = (uint32_t)ml.triangle_count * 3;
        dc.instanceCount = 1;
        dc.firstVertex = 0;
        dc.firstInstance = section_base + slot;
        L.draws()[slot] = dc;
        L.refs[slot] = refs[id];
    }
}

// ------------------------------------------------------------ rasterisation rules
struct ClipV { float x, y, z, w; };
struct SnapV { int32_t X, Y; float z; };

// A vertex with a non-finite coordinate drops the whole triangle.
static bool finite4(const ClipV& v) {
    return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z) && std::isfinite(v.w);
}
// Outcode bits: 1 z > w (or w <= 0), 2 z < 0, 4 x > g*w, 8 x < -g*w,
// 16 y > g*w, 32 y < -g*w.
static uint32_t outcode(const ClipV& v) {
    uint32_t c = 0;
    float g = LH_GUARD_BAND * v.w;
    if (v.z > v.w || !(v.w > 0.0f)) c |= 1;
    if (v.z < 0.0f) c |= 2;
    if (v.x > g) c |= 4;
    if (v.x < -g) c |= 8;
    if (v.y > g) c |= 16;
    if (v.y < -g) c |= 32;
    return c;
}
// Vulkan viewport transform x_f = (w/2) x_d + (x + w/2), y likewise
// (viewport at 0,0 with positive height), snapped to 1/256 pixel.
static SnapV snap(const ClipV& v, float hw, float hh) {
    float ndx = v.x / v.w, ndy = v.y / v.w;
    SnapV s;
    s.z = v.z / v.w;
    float xf = ndx * hw + hw, yf = ndy * hh + hh;
    s.X = (int32_t)std::nearbyint(xf * 256.0f);
    s.Y = (int32_t)std::nearbyint(yf * 256.0f);
    return s;
}
static int64_t edge(const SnapV& a, const SnapV& b, int64_t px, int64_t py) {
    return (int64_t)(b.Y - a.Y) * (px - a.X) - (int64_t)(b.X - a.X) * (py - a.Y);
}
static bool top_left(const SnapV& a, const SnapV& b) {
    int32_t dy = b.Y - a.Y, dx = b.X - a.X;
    return dy > 0 || (dy == 0 && dx < 0);
}

// Alpha test of the alpha-clip pipelines (rasterization.glsl:66-97,
// 118-145): a fragment is discarded when the base-colour texture's alpha,
// sampled bilinearly with repeat addressing at the perspective-correct uv of
// the pixel centre, is below 0.5.  The perspective-correct barycentrics come
// from the 2D homogeneous edge functions of the unclipped triangle (Olano and
// Greer, "Triangle scan conversion using 2D homogeneous coordinates", 1997):
// for clip positions v_k = (x_k, y_k, w_k), E_k(nx, ny) = a_k nx + b_k ny + c_k
// with (a_k, b_k, c_k) = v_i x v_j for (i, j) = (1, 2), (2, 0), (0, 1), and
// lambda_k = E_k / (E_0 + E_1 + E_2) -- which holds for clipped triangles too.
// uv_k = uv(vertex k) * texture_scale + texture_offset, per vertex as the
// reference's vertex shaders form it.
struct AlphaTest {
    float a[3], b[3], c[3];
    float u[3], v[3];
    uint32_t tex;  // base_color_texture_index
};

static AlphaTest alpha_setup(const ClipV c[3], const float u[3], const float v[3], uint32_t tex) {
    AlphaTest t;
    for (int k = 0; k < 3; k++) {
        const ClipV& p = c[(k + 1) % 3];
        const ClipV& q = c[(k + 2) % 3];
        t.a[k] = p.y * q.w - q.y * p.w;
        t.b[k] = p.w * q.x - q.w * p.x;
        t.c[k] = p.x * q.y - q.x * p.y;
        t.u[k] = u[k];
        t.v[k] = v[k];
    }
    t.tex = tex;
    return t;
}

template <class T> struct Tex4 { T r, g, b, a; };
template <class T> static Tex4<T> sample_repeat(const lho_frame_desc* d, uint32_t index, V2<T> uv);

// True when the fragment at pixel (px, py) of a W x H target survives.
static bool alpha_pass(const lho_frame_desc* d, const AlphaTest& t, int32_t px, int32_t py, uint32_t W, uint32_t H) {
    const float nx = (((float)px + 0.5f) / (float)W) * 2.0f - 1.0f;
    const float ny = (((float)py + 0.5f) / (float)H) * 2.0f - 1.0f;
    float e[3];
    for (int k = 0; k < 3; k++) e[k] = (t.a[k] * nx + t.b[k] * ny) + t.c[k];
    const float s = (e[0] + e[1]) + e[2];
    const float l0 = e[0] / s, l1 = e[1] / s, l2 = e[2] / s;
    const float u = (l0 * t.u[0] + l1 * t.u[1]) + l2 * t.u[2];
    const float v = (l0 * t.v[0] + l1 * t.v[1]) + l2 * t.v[2];
    return !(sample_repeat<float>(d, t.tex, V2<float>{u, v}).a < 0.5f);
}

struct Target {
    uint32_t kind;  // 0 visibility (u64 max), 1 shadow depth (u32 min)
    uint32_t W, H;
    uint64_t* vis;
    uint32_t* depth;
    uint32_t id;
    uint64_t* stats;  // per-thread counters (may be null)
    const AlphaTest* alpha = nullptr;  // alpha-clip draw: double sided, alpha tested
    const lho_frame_desc* desc = nullptr;
};

// Rasterise one snapped triangle whose orientation is already normalised
// (cross < 0, interior has all edge functions >= 0).
static void raster_tri(const Target& t, SnapV v0, SnapV v1, SnapV v2) {
    int64_t A = edge(v1, v2, v0.X, v0.Y);  // = twice the area, > 0
    if (A <= 0) return;
    int32_t minX = std::min(v0.X, std::min(v1.X, v2.X)), maxX = std::max(v0.X, std::max(v1.X, v2.X));
    int32_t minY = std::min(v0.Y, std::min(v1.Y, v2.Y)), maxY = std::max(v0.Y, std::max(v1.Y, v2.Y));
    int32_t px0 = (minX + 127) >> 8, px1 = (maxX - 128) >> 8;
    int32_t py0 = (minY + 127) >> 8, py1 = (maxY - 128) >> 8;
    px0 = std::max(px0, 0); py0 = std::max(py0, 0);
    px1 = std::min(px1, (int32_t)t.W - 1); py1 = std::min(py1, (int32_t)t.H - 1);
    if (px0 > px1 || py0 > py1) return;
    if (t.stats) {
        uint64_t npx = (uint64_t)(px1 - px0 + 1) * (uint64_t)(py1 - py0 + 1);
        t.stats[0]++;
        t.stats[npx <= 4 ? 2 : npx <= 64 ? 3 : npx <= 4096 ? 4 : 5]++;
    }
    int64_t b12 = top_left(v1, v2) ? 0 : 1, b20 = top_left(v2, v0) ? 0 : 1, b01 = top_left(v0, v1) ? 0 : 1;
    float fA = (float)A;
    float s1 = (v1.z - v0.z) / fA, s2 = (v2.z - v0.z) / fA;
    for (int32_t py = py0; py <= py1; py++) {
        int64_t Py = (int64_t)py * 256 + 128;
        for (int32_t px = px0; px <= px1; px++) {
            int64_t Px = (int64_t)px * 256 + 128;
            int64_t e12 = edge(v1, v2, Px, Py), e20 = edge(v2, v0, Px, Py), e01 = edge(v0, v1, Px, Py);
            if (e12 < b12 || e20 < b20 || e01 < b01) continue;
            if (t.alpha && !alpha_pass(t.desc, *t.alpha, px, py, t.W, t.H)) continue;
            float dpt = (v0.z + (float)e20 * s1) + (float)e01 * s2;
            dpt = dpt > 0.0f ? dpt : 0.0f;
            dpt = dpt < 1.0f ? dpt : 1.0f;
            if (t.stats) t.stats[1]++;
            size_t pix = (size_t)py * t.W + px;
            if (t.kind == 0)
                atomic_max_u64(&t.vis[pix], ((uint64_t)f2u(dpt) << 32) | t.id);
            else
                atomic_min_u32(&t.depth[pix], f2u(dpt));
        }
    }
}

static int64_t poly_cross(const SnapV* p, int n) {
    int64_t c = 0;
    for (int i = 0; i < n; i++) {
        const SnapV &a = p[i], &b = p[(i + 1) % n];
        c += (int64_t)a.X * b.Y - (int64_t)b.X * a.Y;
    }
    return c;
}

// Fixed-function primitive processing of one triangle: clip (only when a
// vertex leaves the guard band or 0 <= z <= w), viewport transform and
// snapping, face culling (Vulkan area sign, front face = counter-clockwise;
// visibility culls back faces, shadow culls front faces,
// src/pipelines.cpp:10-19,257-300), then coverage and depth.
static void raster_primitive(const Target& t, const ClipV c[3]) {
    if (!finite4(c[0]) || !finite4(c[1]) || !finite4(c[2])) return;
    uint32_t o0 = outcode(c[0]), o1 = outcode(c[1]), o2 = outcode(c[2]);
    if (o0 & o1 & o2) return;
    float hw = (float)t.W * 0.5f, hh = (float)t.H * 0.5f;
    ClipV poly[9];
    int n = 3;
    poly[0] = c[0]; poly[1] = c[1]; poly[2] = c[2];
    if (o0 | o1 | o2) {
        // Sutherland-Hodgman against w-z, z, g*w-x, g*w+x, g*w-y, g*w+y >= 0.
        for (int plane = 0; plane < 6 && n >= 3; plane++) {
            ClipV out[9];
            int m = 0;
            auto dist = [&](const ClipV& v) {
                float g = LH_GUARD_BAND * v.w;
                switch (plane) {
                    case 0: return v.w - v.z;
                    case 1: return v.z;
                    case 2: return g - v.x;
                    case 3: return g + v.x;
                    case 4: return g - v.y;
                    default: return g + v.y;
                }
            };
            for (int i = 0; i < n; i++) {
                const ClipV &a = poly[i], &b = poly[(i + 1) % n];
                float da = dist(a), db = dist(b);
                if (da >= 0.0f) out[m++] = a;
                if ((da >= 0.0f) != (db >= 0.0f)) {
                    float tt = da / (da - db);
                    out[m++] = ClipV{a.x + tt * (b.x - a.x), a.y + tt * (b.y - a.y), a.z + tt * (b.z - a.z),
                                     a.w + tt * (b.w - a.w)};
                }
            }
            n = m;
            for (int i = 0; i < n; i++) poly[i] = out[i];
        }
        if (n < 3) return;
        // a vertex left at w <= 0 (only a triangle through the eye point) cannot be projected
        for (int i = 0; i < n; i++)
            if (!(poly[i].w > 0.0f)) return;
        if (t.stats) t.stats[6]++;
    }
    SnapV s[9];
    for (int i = 0; i < n; i++) s[i] = snap(poly[i], hw, hh);
    int64_t pc = poly_cross(s, n);
    // cross < 0 <=> Vulkan area > 0 <=> counter-clockwise <=> front facing
    if (pc == 0) return;
    if (!t.alpha && t.kind == 0 && pc > 0) return;  // visibility: cull back faces
    if (!t.alpha && t.kind == 1 && pc < 0) return;  // shadow: cull front faces
    // (alpha clip: FILL_RASTERIZATION_DOUBLE_SIDED, pipelines.cpp:272-285,302-315)
    for (int i = 1; i + 1 < n; i++) {
        SnapV a = s[0], b = s[i], d = s[i + 1];
        SnapV tri[3] = {a, b, d};
        int64_t tc = poly_cross(tri, 3);
        if (tc == 0 || ((tc < 0) != (pc < 0))) continue;
        if (tc > 0) std::swap(b, d);
        raster_tri(t, a, b, d);
    }
}

// rasterization.glsl:12-34 (load_vertex_data) for one triangle of a draw.
static bool triangle_clip(const lho_frame_desc* d, const lh_mat4& vp, const MeshletReference& ref, uint32_t tri,
                          ClipV out[3], uint32_t* flags, AlphaTest* alpha = nullptr) {
    const Instance& inst = d->instances[ref.instance_index];
    const MeshInfo& mi = mesh_info_of(inst);
    const Meshlet& ml = meshlet_of(mi, ref.meshlet_index);
    const uint8_t* micro = reinterpret_cast<const uint8_t*>((uintptr_t)mi.micro_indices) + ml.triangle_offset;
    for (int k = 0; k < 3; k++) {
        uint32_t m = micro[tri * 3 + k];
        if (m >= ml.index_count) { *flags |= LH_FLAG_BAD_MESHLET; return false; }
        uint32_t index = load_index(mi, ml.index_offset + m);
        vec3 w = calculate_world_pos<float>(inst, mi, index);
        vec4 c = mul<float>(vp, vec4{w.x, w.y, w.z, 1.0f});
        out[k] = ClipV{c.x, c.y, c.z, c.w};
        if (alpha) {
            V2<float> uv = load_uv_raw<float>(mi, index);
            alpha->u[k] = uv.x * mi.texture_scale.x + mi.texture_offset.x;
            alpha->v[k] = uv.y * mi.texture_scale.y + mi.texture_offset.y;
        }
    }
    if (alpha) *alpha = alpha_setup(out, alpha->u, alpha->v, mi.base_color_texture_index);
    return true;
}

// Visibility or shadow raster of one view: the opaque draws
// (rasterization.glsl:38-58, 101-111 with the state of
// src/pipelines.cpp:257-270,287-300), then the alpha-clip draws, double
// sided and alpha tested (rasterization.glsl:60-97, 113-145;
// pipelines.cpp:272-285,302-315).
static void raster_view(Frame& F, uint32_t view, const Target& tgt_proto, const lh_mat4& vp) {
    ViewLists L = F.lists(view);
    uint32_t md = F.d->max_draws;
    uint32_t nop = std::min(L.num_opaque(), md), nal = std::min(L.num_alpha(), md);
    std::vector<uint32_t> slots;
    for (uint32_t i = 0; i < nop; i++) slots.push_back(i);
    for (uint32_t i = 0; i < nal; i++) slots.push_back(md + i);
    std::atomic<uint32_t> flags{0};
    std::vector<std::atomic<uint64_t>> acc(8);
    uint64_t* out_stats = F.o->stats + (tgt_proto.kind ? 8 : 0);
    F.pool.run(slots.size(), 16, [&](size_t b, size_t e) {
        uint32_t fl = 0;
        uint64_t st[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (size_t k = b; k < e; k++) {
            uint32_t slot = slots[k];
            const MeshletReference& ref = L.refs[slot];
            const Meshlet& ml = meshlet_of(mesh_info_of(F.d->instances[ref.instance_index]), ref.meshlet_index);
            // A meshlet beyond the meshletiser limits (64 vertices, 124
            // triangles; shared_cpu_gpu.h:148-150) is malformed: skipped, flagged.
            if (ml.index_count > MAX_MESHLET_UNIQUE_VERTICES || ml.triangle_count > MAX_MESHLET_TRIANGLES) {
                fl |= LH_FLAG_BAD_MESHLET;
                continue;
            }
            const bool alpha = slot >= md;  // the alpha-clip draw class
            for (uint32_t tri = 0; tri < ml.triangle_count; tri++) {
                ClipV c[3];
                AlphaTest at;
                if (!triangle_clip(F.d, vp, ref, tri, c, &fl, alpha ? &at : nullptr)) continue;
                Target t = tgt_proto;
                t.id = LH_PACK_ID(tri, slot);
                t.stats = st;
                t.alpha = alpha ? &at : nullptr;
                t.desc = F.d;
                raster_primitive(t, c);
            }
            uint64_t frags = st[1] - st[7];
            st[7] = st[1];
            uint64_t cur = acc[7].load();
            while (frags > cur && !acc[7].compare_exchange_weak(cur, frags)) {}
        }
        for (int i = 0; i < 7; i++) acc[i] += st[i];
        flags.fetch_or(fl);
    });
    F.o->flags |= flags.load();
    for (int i = 0; i < 8; i++) out_stats[i] += acc[i].load();
}

// ------------------------------------------------------------ read_depth.glsl
// read_depth.glsl:3-18
static uint32_t min_if_not_zero(uint32_t a, uint32_t b) { return a != 0 ? (b != 0 ? std::min(a, b) : a) : b; }

// read_depth.glsl:22-83: each invocation gathers a 4x4 block at
// coord = id*4 with clamp-to-edge; min over non-zero depth bits, max over all.
static void read_depth(Frame& F) {
    uint32_t W = F.W, H = F.H;
    const uint64_t* vis = F.o->visibility;
    std::atomic<uint32_t> gmin{0xFFFFFFFFu}, gmax{0};
    // dispatch_size(extent, 8*4) workgroups of 8x8 (src/rendering.cpp:289-300),
    // invocations at or beyond the window size return (read_depth.glsl:26-30).
    uint32_t nx = std::min(W, ((W - 1) / 32 + 1) * 8), ny = std::min(H, ((H - 1) / 32 + 1) * 8);
    F.pool.run(ny, 16, [&](size_t b, size_t e) {
        uint32_t mn = 0xFFFFFFFFu, mx = 0;
        for (size_t gy = b; gy < e; gy++)
            for (uint32_t gx = 0; gx < nx; gx++) {
                uint32_t vals[16];
                for (int k = 0; k < 16; k++) {
                    uint32_t x = std::min(gx * 4 + (k & 3), W - 1), y = std::min((uint32_t)gy * 4 + (k >> 2), H - 1);
                    vals[k] = (uint32_t)(vis[(size_t)y * W + x] >> 32);
                }
                uint32_t dmin = 0, dmax = 0;
                for (int k = 0; k < 16; k++) { dmin = min_if_not_zero(dmin, vals[k]); dmax = std::max(dmax, vals[k]); }
                if (dmin != 0) mn = std::min(mn, dmin);
                mx = std::max(mx, dmax);
            }
        uint32_t cur = gmin.load();
        while (mn < cur && !gmin.compare_exchange_weak(cur, mn)) {}
        cur = gmax.load();
        while (mx > cur && !gmax.compare_exchange_weak(cur, mx)) {}
    });
    F.o->misc->min_depth = std::min(F.o->misc->min_depth, gmin.load());
    F.o->misc->max_depth = std::max(F.o->misc->max_depth, gmax.load());
}

// ------------------------------------------------------------ generate_shadow_matrices.glsl
// matrices.glsl:9-19
static lh_mat4 look_at(vec3 eye, vec3 at, vec3 up) {
    vec3 f = normalize(at - eye);
    vec3 r = normalize(cross(f, up));
    vec3 u = cross(r, f);
    lh_mat4 m;
    m.cols[0] = {r.x, u.x, -f.x, 0.0f};
    m.cols[1] = {r.y, u.y, -f.y, 0.0f};
    m.cols[2] = {r.z, u.z, -f.z, 0.0f};
    m.cols[3] = {-dot(r, eye), -dot(u, eye), dot(f, eye), 1.0f};
    return m;
}
// matrices.glsl:21-40
static lh_mat4 orthographic(float left, float right, float bottom, float top, float near_, float far_) {
    float rml = right - left, rpl = right + left, tmb = top - bottom, tpb = top + bottom, fmn = far_ - near_;
    lh_mat4 m;
    m.cols[0] = {2.0f / rml, 0.0f, 0.0f, 0.0f};
    m.cols[1] = {0.0f, -2.0f / tmb, 0.0f, 0.0f};
    m.cols[2] = {0.0f, 0.0f, -1.0f / fmn, 0.0f};
    m.cols[3] = {-(rpl / rml), -(tpb / tmb), -(near_ / fmn), 1.0f};
    return m;
}

// generate_shadow_matrices.glsl:15-110.  pow(0.5, p) and pow(0.75, p) depend
// only on the uniform split exponent; both sides evaluate them on the host
// in double precision and round to float.
static void generate_shadow_matrices(Frame& F) {
    const Uniforms& u = *F.d->uniforms;
    MiscStorage& m = *F.o->misc;
    float min_depth = u2f(m.min_depth), max_depth = u2f(m.max_depth);
    float min_distance = NEAR_PLANE / max_depth;  // util.glsl:23-25
    float max_distance = NEAR_PLANE / min_depth;
    float p05 = (float)std::pow(0.5, (double)u.cascade_split_pow);
    float p075 = (float)std::pow(0.75, (double)u.cascade_split_pow);
    float splits[4] = {max_depth, NEAR_PLANE / (min_distance * (1.0f - p05) + max_distance * p05),
                       NEAR_PLANE / (min_distance * (1.0f - p075) + max_distance * p075), min_depth};
    for (uint32_t c = 0; c < 4; c++) {
        float last = c > 0 ? splits[c - 1] : max_depth;
        float split = splits[c];
        vec3 corners[8] = {{-1.0f, 1.0f, last},  {1.0f, 1.0f, last},  {1.0f, -1.0f, last},  {-1.0f, -1.0f, last},
                           {-1.0f, 1.0f, split}, {1.0f, 1.0f, split}, {1.0f, -1.0f, split}, {-1.0f, -1.0f, split}};
        for (int i = 0; i < 8; i++) {
            vec4 ic = mul<float>(u.inv_perspective_view, vec4{corners[i].x, corners[i].y, corners[i].z, 1.0f});
            corners[i] = vec3{ic.x / ic.w, ic.y / ic.w, ic.z / ic.w};
        }
        vec3 center{0.0f, 0.0f, 0.0f};
        for (int i = 0; i < 8; i++) center = center + corners[i];
        center = center / 8.0f;
        float radius = 0.0f;
        for (int i = 0; i < 8; i++) radius = std::max(radius, length(corners[i] - center));
        radius = std::ceil(radius * 16.0f) / 16.0f;
        vec3 eye = v3<float>(u.sun_dir) * u.shadow_cam_distance + center;
        lh_mat4 view = look_at(eye, center, vec3{0.0f, 1.0f, 0.0f});
        lh_mat4 proj = orthographic(-radius, radius, -radius, radius, 0.0f, u.shadow_cam_distance * 2.0f);
        lh_mat4 mat = matmul(proj, view);
        lh_mat4 bias;
        bias.cols[0] = {0.5f, 0.0f, 0.0f, 0.0f};
        bias.cols[1] = {0.0f, 0.5f, 0.0f, 0.0f};
        bias.cols[2] = {0.0f, 0.0f, 1.0f, 0.0f};
        bias.cols[3] = {0.5f, 0.5f, 0.0f, 1.0f};
        m.shadow_matrices[c] = mat;
        m.uv_space_shadow_matrices[c] = matmul(bias, mat);
        m.shadow_view_matrices[c] = view;
        m.shadow_sphere_radii[c] = radius;
    }
}

// cull_instances.comp:7-27 (view 0) and :31-56 (cascades); appends in
// ascending instance order.
static void cull_instances(Frame& F, bool shadows) {
    const Uniforms& u = *F.d->uniforms;
    uint32_t n = F.d->n_instances;
    uint32_t nv = shadows ? 4 : 1;
    std::vector<uint8_t> keep((size_t)n * nv);
    F.pool.run(n, 1024, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++) {
            const Instance& inst = F.d->instances[i];
            const MeshInfo& mi = mesh_info_of(inst);
            for (uint32_t c = 0; c < nv; c++)
                keep[i * nv + c] = shadows ? !cull_bounding_sphere_shadows(*F.o->misc, inst, mi.bounding_sphere, c)
                                           : !cull_bounding_sphere(u, inst, mi.bounding_sphere);
        }
    });
    for (uint32_t c = 0; c < nv; c++) {
        Sector s = F.sector(shadows ? 1 + c : 0);
        for (uint32_t i = 0; i < n; i++)
            if (keep[(size_t)i * nv + c])
                prefix_sum_inclusive_append(s, F.d->max_instances, i, mesh_info_of(F.d->instances[i]).num_meshlets,
                                            &F.o->flags);
    }
}

// ------------------------------------------------------------ samplers
static float srgb_table[256];
static void init_srgb() {
    for (int i = 0; i < 256; i++) {
        double c = i / 255.0;
        srgb_table[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
}


// Bilinear filtering of level 0 with repeat addressing (the reference's
// repeat_sampler, src/main.cpp:550-560, without mip levels / anisotropy).
template <class T> static Tex4<T> sample_repeat(const lho_frame_desc* d, uint32_t index, V2<T> uv) {
    if (index >= d->n_textures) return {0, 0, 0, 0};
    const lh_texture& t = d->textures[index];
    const uint8_t* tex = reinterpret_cast<const uint8_t*>((uintptr_t)t.texels);
    T u = uv.x * (T)t.width - (T)0.5, v = uv.y * (T)t.height - (T)0.5;
    if (!(std::fabs(u) < (T)1e9)) u = 0;
    if (!(std::fabs(v) < (T)1e9)) v = 0;
    T fu = std::floor(u), fv = std::floor(v);
    T a = u - fu, b = v - fv;
    int64_t i0 = (int64_t)fu, j0 = (int64_t)fv;
    int64_t W = t.width, H = t.height;
    int64_t ia = ((i0 % W) + W) % W, ib = (((i0 + 1) % W) + W) % W;
    int64_t ja = ((j0 % H) + H) % H, jb = (((j0 + 1) % H) + H) % H;
    const float* lin = d->texture_linear ? d->texture_linear[index] : nullptr;
    auto texel = [&](int64_t i, int64_t j) {
        Tex4<T> r;
        if (lin) {
            const float* q = lin + ((size_t)j * W + i) * 4;
            r.r = (T)q[0]; r.g = (T)q[1]; r.b = (T)q[2]; r.a = (T)q[3];
            return r;
        }
        const uint8_t* p = tex + ((size_t)j * W + i) * 4;
        if (t.srgb) { r.r = (T)srgb_table[p[0]]; r.g = (T)srgb_table[p[1]]; r.b = (T)srgb_table[p[2]]; }
        else { r.r = (T)p[0] / (T)255; r.g = (T)p[1] / (T)255; r.b = (T)p[2] / (T)255; }
        r.a = (T)p[3] / (T)255;
        return r;
    };
    Tex4<T> t00 = texel(ia, ja), t10 = texel(ib, ja), t01 = texel(ia, jb), t11 = texel(ib, jb);
    T w00 = ((T)1 - a) * ((T)1 - b), w10 = a * ((T)1 - b), w01 = ((T)1 - a) * b, w11 = a * b;
    Tex4<T> r;
    r.r = ((t00.r * w00 + t10.r * w10) + t01.r * w01) + t11.r * w11;
    r.g = ((t00.g * w00 + t10.g * w10) + t01.g * w01) + t11.g * w11;
    r.b = ((t00.b * w00 + t10.b * w10) + t01.b * w01) + t11.b * w11;
    r.a = ((t00.a * w00 + t10.a * w10) + t01.a * w01) + t11.a * w11;
    return r;
}

// Comparison sampling of the cascade array (src/main.cpp:566-580): linear,
// clamp to edge, compare op LESS (1 when ref < stored depth), layer =
// clamp(round(layer), 0, 3).
template <class T> static T sample_shadow(const float* maps, uint32_t S, V2<T> uv, float layer_f, T ref) {
    int layer = (int)std::nearbyint(layer_f);
    layer = std::min(std::max(layer, 0), 3);
    const float* map = maps + (size_t)layer * S * S;
    T u = uv.x * (T)S - (T)0.5, v = uv.y * (T)S - (T)0.5;
    if (!(std::fabs(u) < (T)1e9)) u = 0;
    if (!(std::fabs(v) < (T)1e9)) v = 0;
    T fu = std::floor(u), fv = std::floor(v);
    T a = u - fu, b = v - fv;
    int64_t i0 = (int64_t)fu, j0 = (int64_t)fv;
    auto cl = [&](int64_t i) { return std::min<int64_t>(std::max<int64_t>(i, 0), (int64_t)S - 1); };
    auto cmp = [&](int64_t i, int64_t j) { return ref < (T)map[(size_t)cl(j) * S + cl(i)] ? (T)1 : (T)0; };
    T c00 = cmp(i0, j0), c10 = cmp(i0 + 1, j0), c01 = cmp(i0, j0 + 1), c11 = cmp(i0 + 1, j0 + 1);
    T w00 = ((T)1 - a) * ((T)1 - b), w10 = a * ((T)1 - b), w01 = ((T)1 - a) * b, w11 = a * b;
    return ((c00 * w00 + c10 * w10) + c01 * w01) + c11 * w11;
}

// ------------------------------------------------------------ resolve (render_geometry.comp)
template <class T> struct Bary { V3<T> lambda, ddx, ddy; };

// vbuffer.glsl:11-63
template <class T> static Bary<T> calc_full_bary(V4<T> p0, V4<T> p1, V4<T> p2, V2<T> ndc, V2<T> win) {
    Bary<T> r;
    V3<T> invW{(T)1 / p0.w, (T)1 / p1.w, (T)1 / p2.w};
    V2<T> n0{p0.x * invW.x, p0.y * invW.x}, n1{p1.x * invW.y, p1.y * invW.y}, n2{p2.x * invW.z, p2.y * invW.z};
    // determinant(float2x2(ndc2 - ndc1, ndc0 - ndc1)), columns a, b: a.x*b.y - b.x*a.y
    V2<T> ca{n2.x - n1.x, n2.y - n1.y}, cb{n0.x - n1.x, n0.y - n1.y};
    T invDet = (T)1 / (ca.x * cb.y - cb.x * ca.y);
    r.ddx = V3<T>{n1.y - n2.y, n2.y - n0.y, n0.y - n1.y} * invDet * invW;
    r.ddy = V3<T>{n2.x - n1.x, n0.x - n2.x, n1.x - n0.x} * invDet * invW;
    T ddxSum = dot(r.ddx, V3<T>{1, 1, 1});
    T ddySum = dot(r.ddy, V3<T>{1, 1, 1});
    V2<T> dv{ndc.x - n0.x, ndc.y - n0.y};
    T interpInvW = (invW.x + dv.x * ddxSum) + dv.y * ddySum;
    T interpW = (T)1 / interpInvW;
    r.lambda.x = interpW * ((invW.x + dv.x * r.ddx.x) + dv.y * r.ddy.x);
    r.lambda.y = interpW * (((T)0 + dv.x * r.ddx.y) + dv.y * r.ddy.y);
    r.lambda.z = interpW * (((T)0 + dv.x * r.ddx.z) + dv.y * r.ddy.z);
    r.ddx = r.ddx * ((T)2 / win.x);
    r.ddy = r.ddy * ((T)2 / win.y);
    ddxSum *= (T)2 / win.x;
    ddySum *= (T)2 / win.y;
    r.ddy = r.ddy * (T)-1;
    ddySum *= (T)-1;
    T interpW_ddx = (T)1 / (interpInvW + ddxSum);
    T interpW_ddy = (T)1 / (interpInvW + ddySum);
    r.ddx = (r.lambda * interpInvW + r.ddx) * interpW_ddx - r.lambda;
    r.ddy = (r.lambda * interpInvW + r.ddy) * interpW_ddy - r.lambda;
    return r;
}
// vbuffer.glsl:65-73 (InterpolateWithDeriv) per component.
template <class T> static V3<T> interp_deriv(const Bary<T>& b, T v0, T v1, T v2) {
    V3<T> m{v0, v1, v2};
    return {dot(m, b.lambda), dot(m, b.ddx), dot(m, b.ddy)};
}

template <class T> static T pow_(T x, T y) { return std::pow(x, y); }

static const float PI_F = 3.14159265358979323846f;

// pbr.glsl:3-96
template <class T> static T F_Schlick1(T u, T f0, T f90) { return f0 + (f90 - f0) * pow_((T)1 - u, (T)5); }
template <class T> static T Fd_Burley(T NoV, T NoL, T LoH, T rough) {
    T f90 = (T)0.5 + (T)2 * rough * LoH * LoH;
    T light = F_Schlick1<T>(NoL, (T)1, f90);
    T view = F_Schlick1<T>(NoV, (T)1, f90);
    return light * view * ((T)1 / (T)PI_F);
}
template <class T> static T D_GGX(T NoH, T a) {
    T a2 = a * a;
    T f = (NoH * a2 - NoH) * NoH + (T)1;
    return a2 / ((T)PI_F * f * f);
}
template <class T> static V3<T> F_Schlick3(T u, V3<T> f0) {
    T p = pow_((T)1 - u, (T)5);
    return {f0.x + ((T)1 - f0.x) * p, f0.y + ((T)1 - f0.y) * p, f0.z + ((T)1 - f0.z) * p};
}
template <class T> static T V_SmithGGXCorrelated(T NoV, T NoL, T a) {
    T a2 = a * a;
    T GGXL = NoV * std::sqrt((-NoL * a2 + NoL) * NoL + a2);
    T GGXV = NoL * std::sqrt((-NoV * a2 + NoV) * NoV + a2);
    return (T)0.5 / (GGXV + GGXL);
}
template <class T> static V3<T> BRDF(V3<T> v, V3<T> l, V3<T> n, T pr, T metallic, V3<T> base, bool thin) {
    V3<T> h = normalize(v + l);
    V3<T> diffuse = base * ((T)1 - metallic);
    T refl = ((T)1.5 - (T)1) / ((T)1.5 + (T)1);
    refl = refl * refl;
    V3<T> f0 = V3<T>{refl, refl, refl} * ((T)1 - metallic) + base * metallic;
    T NoV = clampf(dot(n, v), (T)1e-5, (T)1);
    T NoL = clampf(dot(n, l), (T)0, (T)1);
    T NoH = clampf(dot(n, h), (T)0, (T)1);
    T LoH = clampf(dot(l, h), (T)0, (T)1);
    T rough = pr * pr;
    T D = D_GGX(NoH, rough);
    V3<T> F = F_Schlick3(LoH, f0);
    T V = V_SmithGGXCorrelated(NoV, NoL, rough);
    V3<T> Fr = F * (D * V);
    V3<T> Fd = diffuse * Fd_Burley(NoV, NoL, LoH, rough);
    V3<T> irr = (Fd + Fr) * NoL;
    irr = V3<T>{std::max(irr.x, (T)0), std::max(irr.y, (T)0), std::max(irr.z, (T)0)};
    T rNoV = clampf(dot(-n, v), (T)1e-5, (T)1);
    T rNoL = clampf(dot(-n, l), (T)0, (T)1);
    V3<T> back = diffuse * Fd_Burley(rNoV, rNoL, LoH, rough) * rNoL;
    if (thin) irr = irr + back;
    return {std::isnan(irr.x) ? (T)0 : irr.x, std::isnan(irr.y) ? (T)0 : irr.y, std::isnan(irr.z) ? (T)0 : irr.z};
}

// Procedural sky standing in for the missing cubemap asset
// (render_geometry.comp:86-101 samples hdr-cubemap-1024x1024.dds).
template <class T> static V3<T> sky(V3<T> ray) {
    return {(T)0.25 + (T)0.10 * ray.y, (T)0.35 + (T)0.15 * ray.y, (T)0.55 + (T)0.25 * ray.y};
}

// DEBUG_COLOURS (shaders/common/debug.glsl:1-11).
static const float kDebugColours[10][3] = {
    {0.0f / 255.0f, 2.0f / 255.0f, 91.0f / 255.0f},     {0.0f / 255.0f, 108.0f / 255.0f, 251.0f / 255.0f},
    {0.0f / 255.0f, 221.0f / 255.0f, 221.0f / 255.0f},  {51.0f / 255.0f, 221.0f / 255.0f, 0.0f / 255.0f},
    {255.0f / 255.0f, 252.0f / 255.0f, 0.0f / 255.0f},  {255.0f / 255.0f, 180.0f / 255.0f, 0.0f / 255.0f},
    {255.0f / 255.0f, 104.0f / 255.0f, 0.0f / 255.0f},  {226.0f / 255.0f, 22.0f / 255.0f, 0.0f / 255.0f},
    {191.0f / 255.0f, 0.0f / 255.0f, 83.0f / 255.0f},   {145.0f / 255.0f, 0.0f / 255.0f, 65.0f / 255.0f}};
template <class T> static V3<T> debug_colour(uint32_t i) {
    return {(T)kDebugColours[i][0], (T)kDebugColours[i][1], (T)kDebugColours[i][2]};
}

// render_geometry.comp:70-308 for one pixel.
template <class T> static V4<T> resolve_pixel(const lho_frame_desc* d, const lho_frame_out* o, uint32_t x, uint32_t y) {
    const Uniforms& u = *d->uniforms;
    uint32_t W = u.window_size.x, H = u.window_size.y;
    V2<T> ndc{(T)(float)x / (T)(float)W * (T)2 - (T)1, (T)(float)y / (T)(float)H * (T)2 - (T)1};
    uint64_t vis = o->visibility[(size_t)y * W + x];
    uint32_t depth_bits = (uint32_t)(vis >> 32);
    if (u2f(depth_bits) == 0.0f) {
        V4<T> un = mul<T>(u.perspective_inverse, V4<T>{ndc.x, ndc.y, (T)0, (T)1});
        V3<T> lr = normalize(V3<T>{un.x, un.y, un.z});
        V4<T> r4 = mul<T>(u.view_inverse, V4<T>{lr.x, lr.y, lr.z, (T)0});
        V3<T> s = sky(V3<T>{r4.x, r4.y, r4.z}) * pow_((T)2, (T)3);
        return {s.x, s.y, s.z, (T)1};
    }
    uint32_t packed = (uint32_t)vis;
    uint32_t slot = packed & ((1u << 24) - 1), tri = packed >> 24;
    const MeshletReference& ref = o->meshlet_references[slot];
    const Instance& inst = d->instances[ref.instance_index];
    const MeshInfo& mi = mesh_info_of(inst);
    const Meshlet& ml = meshlet_of(mi, ref.meshlet_index);
    const uint8_t* micro = reinterpret_cast<const uint8_t*>((uintptr_t)mi.micro_indices) + ml.triangle_offset + tri * 3;
    uint32_t idx[3];
    for (int k = 0; k < 3; k++) idx[k] = load_index(mi, ml.index_offset + micro[k]);
    V3<T> pa = calculate_world_pos<T>(inst, mi, idx[0]);
    V3<T> pb = calculate_world_pos<T>(inst, mi, idx[1]);
    V3<T> pc = calculate_world_pos<T>(inst, mi, idx[2]);
    const lh_mat4& PV = u.combined_perspective_view;
    Bary<T> bary = calc_full_bary<T>(mul<T>(PV, V4<T>{pa.x, pa.y, pa.z, (T)1}), mul<T>(PV, V4<T>{pb.x, pb.y, pb.z, (T)1}),
                                     mul<T>(PV, V4<T>{pc.x, pc.y, pc.z, (T)1}), ndc, V2<T>{(T)(float)W, (T)(float)H});
    V3<T> wx = interp_deriv(bary, pa.x, pb.x, pc.x), wy = interp_deriv(bary, pa.y, pb.y, pc.y),
          wz = interp_deriv(bary, pa.z, pb.z, pc.z);
    V3<T> world{wx.x, wy.x, wz.x}, wdx{wx.y, wy.y, wz.y}, wdy{wx.z, wy.z, wz.z};
    V2<T> ts{(T)mi.texture_scale.x, (T)mi.texture_scale.y};
    V2<T> ua = load_uv_raw<T>(mi, idx[0]), ub = load_uv_raw<T>(mi, idx[1]), uc = load_uv_raw<T>(mi, idx[2]);
    V3<T> uvx = interp_deriv(bary, ua.x * ts.x, ub.x * ts.x, uc.x * ts.x);
    V3<T> uvy = interp_deriv(bary, ua.y * ts.y, ub.y * ts.y, uc.y * ts.y);
    V2<T> uv{uvx.x + (T)mi.texture_offset.x, uvy.x + (T)mi.texture_offset.y};
    V2<T> uvdx{uvx.y, uvy.y}, uvdy{uvx.z, uvy.z};
    V3<T> view_vector = normalize(v3<T>(u.camera_pos) - world);
    V3<T> na = normalize(load_normal_raw<T>(mi, idx[0])), nb = normalize(load_normal_raw<T>(mi, idx[1])),
          nc = normalize(load_normal_raw<T>(mi, idx[2]));
    V3<T> normal{interp_deriv(bary, na.x, nb.x, nc.x).x, interp_deriv(bary, na.y, nb.y, nc.y).x,
                 interp_deriv(bary, na.z, nb.z, nc.z).x};
    normal = normalize(mul3<T>(inst.normal_transform, normal));
    V3<T> gn = cross(pb - pa, pc - pa);
    bool back = dot(gn, view_vector) < (T)0;
    if (back) normal = -normal;
    uint32_t ci;
    V4<T> sc{0, 0, 0, 0};
    for (ci = 0; ci < 4; ci++) {
        sc = mul<T>(o->misc->uv_space_shadow_matrices[ci], V4<T>{world.x, world.y, world.z, (T)1});
        T ox = sc.x - (T)0.5, oy = sc.y - (T)0.5;
        if (std::fabs(ox) < (T)0.5 && std::fabs(oy) < (T)0.5) break;
    }
    bool alpha = (mi.flags & MESH_INFO_FLAGS_ALPHA_CLIP) != 0;
    T bias = alpha ? (T)0.000002f : (T)0;
    sc = V4<T>{sc.x / sc.w, sc.y / sc.w, sc.z / sc.w, sc.w / sc.w};
    T shadow_sum = 0;
    for (int ox = -1; ox <= 1; ox++)
        for (int oy = -1; oy <= 1; oy++) {
            V2<T> off{(T)(float)ox / (T)1024, (T)(float)oy / (T)1024};
            shadow_sum += sample_shadow<T>(o->shadow_maps, d->shadow_size, V2<T>{sc.x + off.x, sc.y + off.y}, (float)ci,
                                           sc.z - bias);
        }
    shadow_sum /= (T)9;
    if (sc.z > (T)1) shadow_sum = (T)1;
    Tex4<T> bc = sample_repeat<T>(d, mi.base_color_texture_index, uv);
    V3<T> base{bc.r * (T)mi.base_color_factor.x, bc.g * (T)mi.base_color_factor.y, bc.b * (T)mi.base_color_factor.z};
    Tex4<T> mr = sample_repeat<T>(d, mi.metallic_roughness_texture_index, uv);
    T roughness = mr.g, metallic = mr.b;
    if (mi.normal_texture_index != UNUSED_TEXTURE_INDEX) {
        Tex4<T> nt = sample_repeat<T>(d, mi.normal_texture_index, uv);
        V3<T> mn{nt.r * (T)255 / (T)127 - (T)128 / (T)127, nt.g * (T)255 / (T)127 - (T)128 / (T)127,
                 nt.b * (T)255 / (T)127 - (T)128 / (T)127};
        // render_geometry.comp:25-38 (cotangent frame)
        V3<T> dpy = cross(wdy, normal), dpx = cross(normal, wdx);
        V3<T> t = dpy * uvdx.x + dpx * uvdy.x;
        V3<T> b = dpy * uvdx.y + dpx * uvdy.y;
        T invmax = (T)1 / std::sqrt(std::max(dot(t, t), dot(b, b)));
        V3<T> tt = t * invmax, bb = b * invmax;
        normal = normalize(V3<T>{(tt.x * mn.x + bb.x * mn.y) + normal.x * mn.z, (tt.y * mn.x + bb.y * mn.y) + normal.y * mn.z,
                                 (tt.z * mn.x + bb.z * mn.y) + normal.z * mn.z});
    }
    // render_geometry.comp:40-57: AMBIENT_SH has only sh[0] = sh[2] = 0.025
    T amb_level = (T)0.025f;
    V3<T> zero{0, 0, 0};
    V3<T> sh0{amb_level, amb_level, amb_level}, sh2 = sh0;
    V3<T> amb = ((((((((sh0 + zero * normal.x) + sh2 * normal.y) + zero * normal.z) + zero * (normal.x * normal.z)) +
                     zero * (normal.z * normal.y)) + zero * (normal.y * normal.x)) +
                  zero * ((T)3 * normal.z * normal.z - (T)1)) + zero * (normal.x * normal.x - normal.y * normal.y));
    V3<T> ambient = amb * (base * ((T)1 - metallic));
    T sun_intensity = (T)PI_F * shadow_sum;
    // Uniforms.sun_intensity as the light colour: (1,1,1) reproduces the
    // reference, whose shaders do not read the field (main.cpp:649).
    V3<T> sun = (BRDF<T>(view_vector, v3<T>(u.sun_dir), normal, roughness, metallic, base, alpha) * sun_intensity) *
                v3<T>(u.sun_intensity);
    V3<T> out = sun + ambient;
    // debug views (render_geometry.comp:268-308); the shader-clock heat map
    // measures time and has no CPU counterpart (left as the lit colour)
    switch (u.debug) {
        case 1: out = base * debug_colour<T>(ci); break;                // UNIFORMS_DEBUG_CASCADES
        case 2: out = debug_colour<T>(tri % 10); break;                 // UNIFORMS_DEBUG_TRIANGLE_INDEX
        case 3: out = debug_colour<T>(ref.meshlet_index % 10); break;   // UNIFORMS_DEBUG_INSTANCE_INDEX
        case 5: out = normal * (T)0.5 + V3<T>{(T)0.5, (T)0.5, (T)0.5}; break;  // UNIFORMS_DEBUG_NORMALS
        default: break;
    }
    return {out.x, out.y, out.z, (T)1};
}

static void render_geometry(Frame& F) {
    uint32_t W = F.W, H = F.H;
    F.pool.run(H, 4, [&](size_t b, size_t e) {
        for (size_t y = b; y < e; y++)
            for (uint32_t x = 0; x < W; x++) {
                V4<float> c = resolve_pixel<float>(F.d, F.o, x, (uint32_t)y);
                float* p = F.o->hdr + ((size_t)y * W + x) * 4;
                p[0] = c.x; p[1] = c.y; p[2] = c.z; p[3] = c.w;
            }
    });
}

static double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

int lho_frame(const lho_frame_desc* d, lho_frame_out* o) {
    if (!d || !o || !d->uniforms || !o->prefix_sums || !o->meshlet_references || !o->draw_calls || !o->visibility ||
        !o->misc)
        return LH_ERR_INVALID_ARGUMENT;
    init_srgb();
    Frame F(d, o);
    uint32_t st = d->stages ? d->stages : LHO_STAGE_ALL;
    double t0 = now_ms(), t = t0;
    std::memset(o->stage_ms, 0, sizeof(o->stage_ms));
    std::memset(o->stats, 0, sizeof(o->stats));
    o->flags = 0;
    // reset_buffers.glsl:9-29 and reset_counters (util.glsl:61-70)
    for (uint32_t v = 0; v < 5; v++) {
        std::memset(F.sector(v).base, 0, 8);
        std::memset(F.lists(v).draw_section, 0, 8);
    }
    o->misc->min_depth = 0xFFFFFFFFu;
    o->misc->max_depth = 0;
    std::memset(o->visibility, 0, sizeof(uint64_t) * F.W * F.H);
    if (o->shadow_maps)
        for (size_t i = 0; i < (size_t)4 * F.S * F.S; i++) o->shadow_maps[i] = 1.0f;
    auto lap = [&](int k) { double n = now_ms(); o->stage_ms[k] += n - t; t = n; };
    if (st & LHO_STAGE_CULL) {
        cull_instances(F, false);
        write_draw_calls(F, 0);
    }
    lap(0);
    if (st & LHO_STAGE_RASTER) {
        Target tg{0, F.W, F.H, o->visibility, nullptr, 0, nullptr};
        raster_view(F, 0, tg, d->uniforms->combined_perspective_view);
    }
    lap(1);
    if (st & LHO_STAGE_DEPTH) {
        read_depth(F);
        if (o->misc->min_depth == 0xFFFFFFFFu) o->flags |= LH_FLAG_NO_DEPTH;
        generate_shadow_matrices(F);
    }
    lap(2);
    if ((st & LHO_STAGE_SHADOW) && o->shadow_maps) {
        cull_instances(F, true);
        for (uint32_t c = 0; c < 4; c++) write_draw_calls(F, 1 + c);
        lap(3);
        for (uint32_t c = 0; c < 4; c++) {
            Target tg{1, F.S, F.S, nullptr, reinterpret_cast<uint32_t*>(o->shadow_maps + (size_t)c * F.S * F.S), 0,
                      nullptr};
            raster_view(F, 1 + c, tg, o->misc->shadow_matrices[c]);
        }
        lap(4);
    }
    if ((st & LHO_STAGE_RESOLVE) && o->hdr && o->shadow_maps) render_geometry(F);
    lap(5);
    o->stage_ms[6] = now_ms() - t0;
    o->stage_ms[7] = (double)F.pool.n;
    return LH_OK;
}

int lho_raster_triangle(const float clip[12], uint32_t id, uint32_t kind, uint32_t width, uint32_t height,
                        uint64_t* target) {
    if (!clip || !target || width == 0 || height == 0 || kind > 1) return LH_ERR_INVALID_ARGUMENT;
    ClipV c[3];
    for (int k = 0; k < 3; k++) c[k] = ClipV{clip[k * 4], clip[k * 4 + 1], clip[k * 4 + 2], clip[k * 4 + 3]};
    Target t{kind, width, height, nullptr, nullptr, id, nullptr};
    std::vector<uint32_t> depth;
    if (kind == 0) {
        t.vis = target;
    } else {
        depth.resize((size_t)width * height);
        for (size_t i = 0; i < depth.size(); i++) depth[i] = (uint32_t)target[i];
        t.depth = depth.data();
    }
    raster_primitive(t, c);
    if (kind == 1)
        for (size_t i = 0; i < depth.size(); i++) target[i] = depth[i];
    return LH_OK;
}

int lho_raster_triangle_alpha(const float clip[12], const float uv[6], const lh_texture* texture, uint32_t id,
                              uint32_t kind, uint32_t width, uint32_t height, uint64_t* target) {
    if (!clip || !uv || !texture || !target || width == 0 || height == 0 || kind > 1) return LH_ERR_INVALID_ARGUMENT;
    init_srgb();
    ClipV c[3];
    for (int k = 0; k < 3; k++) c[k] = ClipV{clip[k * 4], clip[k * 4 + 1], clip[k * 4 + 2], clip[k * 4 + 3]};
    const float u[3] = {uv[0], uv[2], uv[4]}, v[3] = {uv[1], uv[3], uv[5]};
    lho_frame_desc d;
    std::memset(&d, 0, sizeof(d));
    d.textures = texture;
    d.n_textures = 1;
    const AlphaTest at = alpha_setup(c, u, v, 0);
    Target t{kind, width, height, nullptr, nullptr, id, nullptr};
    t.alpha = &at;
    t.desc = &d;
    std::vector<uint32_t> depth;
    if (kind == 0) {
        t.vis = target;
    } else {
        depth.resize((size_t)width * height);
        for (size_t i = 0; i < depth.size(); i++) depth[i] = (uint32_t)target[i];
        t.depth = depth.data();
    }
    raster_primitive(t, c);
    if (kind == 1)
        for (size_t i = 0; i < depth.size(); i++) target[i] = depth[i];
    return LH_OK;
}

// ------------------------------------------------------------ display transform
// display_transform.comp:5-81.  Trilinear LUT sampling with clamp to edge
// (clamp_sampler, main.cpp:561-566), lerped along x, then y, then z.
static void lut_sample(const float* lut, const float uvw[3], float out[3]) {
    const int N = 48;
    float a[3];
    int i0[3], i1[3];
    for (int k = 0; k < 3; k++) {
        float t = uvw[k] * (float)N - 0.5f;
        float fl = std::floor(t);
        a[k] = t - fl;
        int i = (int)fl;
        i0[k] = std::min(std::max(i, 0), N - 1);
        i1[k] = std::min(std::max(i + 1, 0), N - 1);
    }
    auto t = [&](int x, int y, int z, int c) { return lut[(((size_t)z * N + y) * N + x) * 4 + c]; };
    for (int c = 0; c < 3; c++) {
        float c00 = t(i0[0], i0[1], i0[2], c) * (1.0f - a[0]) + t(i1[0], i0[1], i0[2], c) * a[0];
        float c10 = t(i0[0], i1[1], i0[2], c) * (1.0f - a[0]) + t(i1[0], i1[1], i0[2], c) * a[0];
        float c01 = t(i0[0], i0[1], i1[2], c) * (1.0f - a[0]) + t(i1[0], i0[1], i1[2], c) * a[0];
        float c11 = t(i0[0], i1[1], i1[2], c) * (1.0f - a[0]) + t(i1[0], i1[1], i1[2], c) * a[0];
        float c0 = c00 * (1.0f - a[1]) + c10 * a[1], c1 = c01 * (1.0f - a[1]) + c11 * a[1];
        out[c] = c0 * (1.0f - a[2]) + c1 * a[2];
    }
}

static float srgb_oetf(float v) { return v <= 0.003130f ? v * 12.92f : 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f; }

static uint8_t unorm8(float v) {
    v = v > 0.0f ? v : 0.0f;
    v = v < 1.0f ? v : 1.0f;
    return (uint8_t)std::floor(v * 255.0f + 0.5f);
}

int lho_display_transform(const float* hdr, uint32_t W, uint32_t H, const float* lut, const float* shadow_maps,
                          uint32_t S, uint32_t debug_shadowmaps, uint8_t* out) {
    if (!hdr || !out || (debug_shadowmaps && (!shadow_maps || !S))) return LH_ERR_INVALID_ARGUMENT;
    std::vector<float> identity;
    if (!lut) {
        identity.resize(48 * 48 * 48 * 4);
        for (int z = 0; z < 48; z++)
            for (int y = 0; y < 48; y++)
                for (int x = 0; x < 48; x++) {
                    float* p = &identity[(((size_t)z * 48 + y) * 48 + x) * 4];
                    p[0] = x / 47.0f;
                    p[1] = y / 47.0f;
                    p[2] = z / 47.0f;
                    p[3] = 1.0f;
                }
        lut = identity.data();
    }
    const float scale = (48.0f - 1.0f) / 48.0f, bias = 0.5f / 48.0f;
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            const float* s = hdr + ((size_t)y * W + x) * 4;
            float uvw[3], v[3];
            for (int c = 0; c < 3; c++) uvw[c] = (s[c] / (s[c] + 1.0f)) * scale + bias;
            lut_sample(lut, uvw, v);
            if (debug_shadowmaps) {
                const float uvx = ((float)x + 0.5f) / (float)W, uvy = ((float)y + 0.5f) / (float)H;
                const float pct = 0.5f;
                if (uvx < pct && uvy < pct) {
                    const float sx = uvx * 2.0f / pct, sy = uvy * 2.0f / pct;
                    const uint32_t cascade = (sy > 1.0f ? 2u : 0u) + (sx > 1.0f ? 1u : 0u);
                    const float* m = shadow_maps + (size_t)cascade * S * S;
                    const float u = sx - std::floor(sx), w = sy - std::floor(sy);
                    const float tu = u * (float)S - 0.5f, tv = w * (float)S - 0.5f;
                    const float fu = std::floor(tu), fv = std::floor(tv);
                    const float a = tu - fu, b = tv - fv;
                    auto cl = [&](int i) { return std::min(std::max(i, 0), (int)S - 1); };
                    const int i0 = cl((int)fu), i1 = cl((int)fu + 1), j0 = cl((int)fv), j1 = cl((int)fv + 1);
                    const float t00 = m[(size_t)j0 * S + i0], t10 = m[(size_t)j0 * S + i1],
                                t01 = m[(size_t)j1 * S + i0], t11 = m[(size_t)j1 * S + i1];
                    const float d = ((t00 * ((1.0f - a) * (1.0f - b)) + t10 * (a * (1.0f - b))) + t01 * ((1.0f - a) * b)) +
                                    t11 * (a * b);
                    const float g = (d - 0.5f) * 100.0f + 0.5f;
                    v[0] = v[1] = v[2] = g;
                }
            }
            uint8_t* o = out + ((size_t)y * W + x) * 4;
            for (int c = 0; c < 3; c++) o[c] = unorm8(srgb_oetf(v[c]));
            o[3] = 255;
        }
    return LH_OK;
}

int lho_resolve_f64(const lho_frame_desc* d, const lho_frame_out* in, double* hdr64) {
    if (!d || !in || !hdr64) return LH_ERR_INVALID_ARGUMENT;
    init_srgb();
    uint32_t W = d->uniforms->window_size.x, H = d->uniforms->window_size.y;
    Pool pool(d->threads);
    pool.run(H, 4, [&](size_t b, size_t e) {
        for (size_t y = b; y < e; y++)
            for (uint32_t x = 0; x < W; x++) {
                V4<double> c = resolve_pixel<double>(d, in, x, (uint32_t)y);
                double* p = hdr64 + ((size_t)y * W + x) * 4;
                p[0] = c.x; p[1] = c.y; p[2] = c.z; p[3] = c.w;
            }
    });
    return LH_OK;
}

int lho_resolve_f64_pixels(const lho_frame_desc* d, const lho_frame_out* in, const uint32_t* xy, uint32_t n,
                           double* hdr64) {
    if (!d || !in || !hdr64 || (n && !xy)) return LH_ERR_INVALID_ARGUMENT;
    init_srgb();
    const uint32_t W = d->uniforms->window_size.x, H = d->uniforms->window_size.y;
    for (uint32_t i = 0; i < n; i++)
        if (xy[2 * i] >= W || xy[2 * i + 1] >= H) return LH_ERR_INVALID_ARGUMENT;
    Pool pool(d->threads);
    pool.run(n, 16, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++) {
            V4<double> c = resolve_pixel<double>(d, in, xy[2 * i], xy[2 * i + 1]);
            double* p = hdr64 + i * 4;
            p[0] = c.x; p[1] = c.y; p[2] = c.z; p[3] = c.w;
        }
    });
    return LH_OK;
}

}  // extern "C"
