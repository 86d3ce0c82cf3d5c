// Seeded synthetic scenes: procedural meshes, meshletiser, bounds, materials,
// instance placement, cameras, and the device upload.  Host code only.
//
// Layouts follow the reference's loader: MeshInfo filled as at
// src/resources/mesh_loading.cpp:660-697, meshlets as at
// src/resources/meshlets.cpp:87-115, instances as at src/main.cpp:433-440.
#include "lh/scene.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------- random
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {  // splitmix64
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double normal() {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

// ---------------------------------------------------------------- small math (host)
struct V3 { double x, y, z; };
static V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
static double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static double len(V3 a) { return std::sqrt(dot(a, a)); }
static V3 norm(V3 a) { double l = len(a); return l > 0 ? a * (1.0 / l) : V3{0, 0, 0}; }

// 4x4 column-major double matrix, m[c][r].
struct M4 { double m[4][4]; };
static M4 identity() { M4 r{}; for (int i = 0; i < 4; i++) r.m[i][i] = 1; return r; }
static M4 mul(const M4& a, const M4& b) {
    M4 r{};
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a.m[k][rr] * b.m[c][k];
            r.m[c][rr] = s;
        }
    return r;
}
static M4 inverse(const M4& a) {
    // Gauss-Jordan on the row-major view of the matrix.
    double t[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) { t[r][c] = a.m[c][r]; t[r][c + 4] = (r == c); }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(t[r][col]) > std::fabs(t[piv][col])) piv = r;
        for (int c = 0; c < 8; c++) std::swap(t[col][c], t[piv][c]);
        double d = t[col][col];
        if (d == 0) return identity();
        for (int c = 0; c < 8; c++) t[col][c] /= d;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            double f = t[r][col];
            if (f != 0)
                for (int c = 0; c < 8; c++) t[r][c] -= f * t[col][c];
        }
    }
    M4 r{};
    for (int rr = 0; rr < 4; rr++)
        for (int c = 0; c < 4; c++) r.m[c][rr] = t[rr][c + 4];
    return r;
}
static lh_mat4 to_f(const M4& a) {
    lh_mat4 r;
    for (int c = 0; c < 4; c++) {
        r.cols[c].x = (float)a.m[c][0]; r.cols[c].y = (float)a.m[c][1];
        r.cols[c].z = (float)a.m[c][2]; r.cols[c].w = (float)a.m[c][3];
    }
    return r;
}
static M4 from_f(const lh_mat4& a) {
    M4 r;
    for (int c = 0; c < 4; c++) {
        r.m[c][0] = a.cols[c].x; r.m[c][1] = a.cols[c].y; r.m[c][2] = a.cols[c].z; r.m[c][3] = a.cols[c].w;
    }
    return r;
}

// glm::lookAt (right handed), the same matrix as src/shaders/common/matrices.glsl:9-19.
static M4 look_at(V3 eye, V3 center, V3 up) {
    V3 f = norm(center - eye);
    V3 s = norm(cross(f, up));
    V3 u = cross(s, f);
    M4 r = identity();
    r.m[0][0] = s.x; r.m[1][0] = s.y; r.m[2][0] = s.z;
    r.m[0][1] = u.x; r.m[1][1] = u.y; r.m[2][1] = u.z;
    r.m[0][2] = -f.x; r.m[1][2] = -f.y; r.m[2][2] = -f.z;
    r.m[3][0] = -dot(s, eye); r.m[3][1] = -dot(u, eye); r.m[3][2] = dot(f, eye);
    return r;
}

// src/projection.h:3-20, evaluated in float as the reference does.
static M4 infinite_reverse_z_perspective(float fov_rad, float width, float height, float near_) {
    float focal_length = 1.0f / std::tan(fov_rad / 2.0f);
    float x = focal_length / (width / height);
    float y = -focal_length;
    M4 r{};
    r.m[0][0] = x;
    r.m[1][1] = y;
    r.m[2][3] = -1.0f;
    r.m[3][2] = near_;
    return r;
}

// ---------------------------------------------------------------- value noise
static uint32_t hash3(int x, int y, int z, uint32_t seed) {
    uint32_t h = seed ^ 0x27d4eb2du;
    h ^= (uint32_t)x * 0x85ebca6bu; h = (h << 13) | (h >> 19);
    h ^= (uint32_t)y * 0xc2b2ae35u; h = (h << 11) | (h >> 21);
    h ^= (uint32_t)z * 0x165667b1u;
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
    return h;
}
static double lattice(int x, int y, int z, uint32_t seed) { return (hash3(x, y, z, seed) & 0xFFFFFF) / 16777215.0; }
static double smooth(double t) { return t * t * (3 - 2 * t); }
static double noise3(double x, double y, double z, uint32_t seed) {
    int ix = (int)std::floor(x), iy = (int)std::floor(y), iz = (int)std::floor(z);
    double fx = smooth(x - ix), fy = smooth(y - iy), fz = smooth(z - iz);
    double v = 0;
    for (int dz = 0; dz < 2; dz++)
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                double w = (dx ? fx : 1 - fx) * (dy ? fy : 1 - fy) * (dz ? fz : 1 - fz);
                v += w * lattice(ix + dx, iy + dy, iz + dz, seed);
            }
    return v;
}
// Periodic 2D value noise on a `period` lattice (tileable textures).
static double noise2p(double x, double y, int period, uint32_t seed) {
    int ix = (int)std::floor(x), iy = (int)std::floor(y);
    double fx = smooth(x - ix), fy = smooth(y - iy);
    auto L = [&](int a, int b) {
        a = ((a % period) + period) % period; b = ((b % period) + period) % period;
        return lattice(a, b, 0, seed);
    };
    return (L(ix, iy) * (1 - fx) + L(ix + 1, iy) * fx) * (1 - fy) + (L(ix, iy + 1) * (1 - fx) + L(ix + 1, iy + 1) * fx) * fy;
}

// ---------------------------------------------------------------- meshes
struct RawMesh {
    std::vector<V3> pos, nrm;
    std::vector<double> u, v;
    std::vector<uint32_t> tris;  // 3 per triangle, emission order (spatially coherent)
};

static void compute_vertex_normals(RawMesh& m) {
    m.nrm.assign(m.pos.size(), V3{0, 0, 0});
    for (size_t t = 0; t + 2 < m.tris.size(); t += 3) {
        V3 a = m.pos[m.tris[t]], b = m.pos[m.tris[t + 1]], c = m.pos[m.tris[t + 2]];
        V3 n = cross(b - a, c - a);
        for (int k = 0; k < 3; k++) m.nrm[m.tris[t + k]] = m.nrm[m.tris[t + k]] + n;
    }
    for (auto& n : m.nrm) { n = norm(n); if (len(n) == 0) n = V3{0, 1, 0}; }
}

// Icosphere: 20 faces subdivided `levels` times, triangles emitted in
// depth-first recursion order so that consecutive triangles are adjacent.
static RawMesh icosphere(int levels) {
    RawMesh m;
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    V3 base[12] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                   {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    int faces[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                        {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                        {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    for (auto& b : base) m.pos.push_back(norm(b));
    std::unordered_map<uint64_t, uint32_t> mid;
    auto midpoint = [&](uint32_t a, uint32_t b) {
        uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        auto it = mid.find(key);
        if (it != mid.end()) return it->second;
        uint32_t id = (uint32_t)m.pos.size();
        m.pos.push_back(norm(m.pos[a] + m.pos[b]));
        mid.emplace(key, id);
        return id;
    };
    struct Rec {
        static void go(RawMesh& m, decltype(midpoint)& mp, uint32_t a, uint32_t b, uint32_t c, int lvl) {
            if (lvl == 0) { m.tris.push_back(a); m.tris.push_back(b); m.tris.push_back(c); return; }
            uint32_t ab = mp(a, b), bc = mp(b, c), ca = mp(c, a);
            go(m, mp, a, ab, ca, lvl - 1);
            go(m, mp, ab, bc, ca, lvl - 1);
            go(m, mp, ab, b, bc, lvl - 1);
            go(m, mp, ca, bc, c, lvl - 1);
        }
    };
    for (auto& f : faces) Rec::go(m, midpoint, (uint32_t)f[0], (uint32_t)f[1], (uint32_t)f[2], levels);
    m.nrm = m.pos;
    for (auto& p : m.pos) {
        m.u.push_back(std::atan2(p.z, p.x) / 6.283185307179586 + 0.5);
        m.v.push_back(std::acos(std::max(-1.0, std::min(1.0, p.y))) / 3.141592653589793);
    }
    return m;
}

// Emit the quads of an (nu x nv) vertex grid in 7x7 blocks; `idx(i, j)`
// gives the vertex id of grid point (i, j).
template <class F>
static void emit_grid(RawMesh& m, int nu, int nv, F idx) {
    const int B = 7;
    for (int bj = 0; bj < nv; bj += B)
        for (int bi = 0; bi < nu; bi += B)
            for (int j = bj; j < std::min(bj + B, nv); j++)
                for (int i = bi; i < std::min(bi + B, nu); i++) {
                    uint32_t a = idx(i, j), b = idx(i + 1, j), c = idx(i + 1, j + 1), d = idx(i, j + 1);
                    m.tris.insert(m.tris.end(), {a, b, c, a, c, d});
                }
}

// Cube-based grid: 6 faces of n x n quads.  `sphere`: project to the unit
// sphere and displace by value noise; else a box with flat faces.
static RawMesh cube_mesh(int n, bool sphere, double amp, uint32_t seed, V3 half) {
    RawMesh m;
    // face frames: origin corner, u axis, v axis (u x v = outward normal)
    struct F { V3 o, du, dv; };
    F faces[6] = {{{1, -1, 1}, {0, 0, -2}, {0, 2, 0}},  {{-1, -1, -1}, {0, 0, 2}, {0, 2, 0}},
                  {{-1, 1, 1}, {2, 0, 0}, {0, 0, -2}},  {{-1, -1, -1}, {2, 0, 0}, {0, 0, 2}},
                  {{-1, -1, 1}, {2, 0, 0}, {0, 2, 0}},  {{1, -1, -1}, {-2, 0, 0}, {0, 2, 0}}};
    for (int f = 0; f < 6; f++) {
        uint32_t base = (uint32_t)m.pos.size();
        V3 fn = norm(cross(faces[f].du, faces[f].dv));
        for (int j = 0; j <= n; j++)
            for (int i = 0; i <= n; i++) {
                double s = (double)i / n, t = (double)j / n;
                V3 p = faces[f].o + faces[f].du * s + faces[f].dv * t;
                if (sphere) {
                    V3 d = norm(p);
                    double r = 1.0 + amp * (noise3(d.x * 3 + 7, d.y * 3 + 3, d.z * 3 + 1, seed) - 0.5) +
                               0.5 * amp * (noise3(d.x * 9, d.y * 9, d.z * 9, seed + 1) - 0.5);
                    p = d * r;
                } else {
                    p = V3{p.x * half.x, p.y * half.y, p.z * half.z};
                }
                m.pos.push_back(p);
                m.nrm.push_back(fn);
                m.u.push_back(s);
                m.v.push_back(t);
            }
        emit_grid(m, n, n, [&](int i, int j) { return base + (uint32_t)(j * (n + 1) + i); });
    }
    if (sphere) compute_vertex_normals(m);
    return m;
}

static RawMesh torus(int nu, int nv, double R, double r) {
    RawMesh m;
    for (int j = 0; j < nv; j++)
        for (int i = 0; i < nu; i++) {
            double a = 6.283185307179586 * i / nu, b = 6.283185307179586 * j / nv;
            V3 c{R * std::cos(a), 0, R * std::sin(a)};
            V3 n{std::cos(b) * std::cos(a), std::sin(b), std::cos(b) * std::sin(a)};
            m.pos.push_back(c + n * r);
            m.nrm.push_back(n);
            m.u.push_back((double)i / nu * 4.0);
            m.v.push_back((double)j / nv);
        }
    // wound so that (b-a)x(c-a) points outward
    emit_grid(m, nu, nv, [&](int i, int j) { return (uint32_t)((j % nv) * nu + (i % nu)); });
    for (size_t t = 0; t < m.tris.size(); t += 3) std::swap(m.tris[t + 1], m.tris[t + 2]);
    return m;
}

// Long thin slivers: a fan of needle triangles (aspect > 100) on a disc.
static RawMesh slivers(int n_tris, uint32_t seed) {
    RawMesh m;
    Rng rng(seed);
    for (int t = 0; t < n_tris; t++) {
        double a = rng.uniform(0, 6.283185307179586), h = rng.uniform(-1, 1);
        V3 d{std::cos(a), 0, std::sin(a)};
        V3 side{-d.z, 0, d.x};
        V3 p0 = V3{0, h, 0} + side * 0.004, p1 = V3{0, h, 0} - side * 0.004, p2 = d * 1.5 + V3{0, h, 0};
        uint32_t b = (uint32_t)m.pos.size();
        m.pos.push_back(p0); m.pos.push_back(p1); m.pos.push_back(p2);
        V3 n = norm(cross(p1 - p0, p2 - p0));
        if (n.y < 0) { std::swap(m.pos[b + 1], m.pos[b + 2]); n = n * -1.0; }
        for (int k = 0; k < 3; k++) { m.nrm.push_back(n); m.u.push_back(k == 2); m.v.push_back(k == 1); }
        m.tris.insert(m.tris.end(), {b, b + 1, b + 2});
    }
    return m;
}

// ---------------------------------------------------------------- bounds
// Ritter-style sphere: the algorithm of src/resources/bounding_sphere.h:3-74
// (which adapts meshoptimizer's): extreme points per axis, the widest pair as
// the initial diameter, then grow to include every point.
static void ritter_sphere(const std::vector<const float*>& pts, float out[4]) {
    size_t n = pts.size();
    size_t pmin[3] = {0, 0, 0}, pmax[3] = {0, 0, 0};
    for (size_t i = 0; i < n; i++)
        for (int a = 0; a < 3; a++) {
            if (pts[i][a] < pts[pmin[a]][a]) pmin[a] = i;
            if (pts[i][a] > pts[pmax[a]][a]) pmax[a] = i;
        }
    float best = 0; int axis = 0;
    for (int a = 0; a < 3; a++) {
        const float *p1 = pts[pmin[a]], *p2 = pts[pmax[a]];
        float d2 = (p2[0] - p1[0]) * (p2[0] - p1[0]) + (p2[1] - p1[1]) * (p2[1] - p1[1]) + (p2[2] - p1[2]) * (p2[2] - p1[2]);
        if (d2 > best) { best = d2; axis = a; }
    }
    const float *p1 = pts[pmin[axis]], *p2 = pts[pmax[axis]];
    float c[3] = {(p1[0] + p2[0]) / 2, (p1[1] + p2[1]) / 2, (p1[2] + p2[2]) / 2};
    float r = std::sqrt(best) / 2;
    for (size_t i = 0; i < n; i++) {
        const float* p = pts[i];
        float d2 = (p[0] - c[0]) * (p[0] - c[0]) + (p[1] - c[1]) * (p[1] - c[1]) + (p[2] - c[2]) * (p[2] - c[2]);
        if (d2 > r * r) {
            float d = std::sqrt(d2);
            float k = 0.5f + (r / d) / 2;
            for (int a = 0; a < 3; a++) c[a] = c[a] * k + p[a] * (1 - k);
            r = (r + d) / 2;
        }
    }
    // Guard against float rounding leaving a point a hair outside.
    float r2 = r;
    for (size_t i = 0; i < n; i++) {
        const float* p = pts[i];
        double d = std::sqrt((double)(p[0] - c[0]) * (p[0] - c[0]) + (double)(p[1] - c[1]) * (p[1] - c[1]) +
                             (double)(p[2] - c[2]) * (p[2] - c[2]));
        if (d > r2) r2 = (float)d;
    }
    out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = r2 * 1.0001f;
}

// ---------------------------------------------------------------- built mesh
struct BuiltMesh {
    // attribute buffers in the layout the shaders read
    std::vector<uint8_t> positions, normals, uvs, indices, micro;
    std::vector<Meshlet> meshlets;
    uint32_t flags = 0;
    uint32_t n_vertices = 0, n_triangles = 0;
    float bounding_sphere[4];
    float tex_scale[2] = {1, 1};
    M4 dequant = identity();  // quantized position -> mesh space
};

static BuiltMesh build_mesh(const RawMesh& raw, bool quantized) {
    BuiltMesh bm;
    size_t nv = raw.pos.size();
    bm.n_vertices = (uint32_t)nv;
    bm.n_triangles = (uint32_t)(raw.tris.size() / 3);
    // Shader-space positions (float) used for every bound.
    std::vector<float> sp(nv * 3);
    if (!quantized) {
        bm.flags |= MESH_INFO_FLAGS_FP32_VERTICES | MESH_INFO_FLAGS_32_BIT_INDICES;
        bm.positions.resize(nv * 12);
        bm.normals.resize(nv * 12);
        bm.uvs.resize(nv * 8);
        for (size_t i = 0; i < nv; i++) {
            float p[3] = {(float)raw.pos[i].x, (float)raw.pos[i].y, (float)raw.pos[i].z};
            float n[3] = {(float)raw.nrm[i].x, (float)raw.nrm[i].y, (float)raw.nrm[i].z};
            float uv[2] = {(float)raw.u[i], (float)raw.v[i]};
            std::memcpy(&bm.positions[i * 12], p, 12);
            std::memcpy(&bm.normals[i * 12], n, 12);
            std::memcpy(&bm.uvs[i * 8], uv, 8);
            std::memcpy(&sp[i * 3], p, 12);
        }
    } else {
        // KHR_mesh_quantization style: u16 positions with the dequantisation
        // folded into the instance transform, i8 normals, u16 uvs.
        V3 lo{1e30, 1e30, 1e30}, hi{-1e30, -1e30, -1e30};
        for (auto& p : raw.pos) {
            lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
            hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
        }
        V3 ext = hi - lo;
        double e = std::max(ext.x, std::max(ext.y, ext.z));
        if (e <= 0) e = 1;
        bm.dequant = identity();
        bm.dequant.m[0][0] = bm.dequant.m[1][1] = bm.dequant.m[2][2] = e / 65535.0;
        bm.dequant.m[3][0] = lo.x; bm.dequant.m[3][1] = lo.y; bm.dequant.m[3][2] = lo.z;
        bm.positions.resize(nv * 6);
        bm.normals.resize(nv * 3);
        bm.uvs.resize(nv * 4);
        double umax = 1;
        for (size_t i = 0; i < nv; i++) umax = std::max(umax, std::max(raw.u[i], raw.v[i]));
        bm.tex_scale[0] = bm.tex_scale[1] = (float)(umax / 65535.0);
        for (size_t i = 0; i < nv; i++) {
            uint16_t q[3];
            double c[3] = {raw.pos[i].x - lo.x, raw.pos[i].y - lo.y, raw.pos[i].z - lo.z};
            for (int a = 0; a < 3; a++) {
                q[a] = (uint16_t)std::lround(std::min(65535.0, std::max(0.0, c[a] / e * 65535.0)));
                sp[i * 3 + a] = (float)q[a];
            }
            std::memcpy(&bm.positions[i * 6], q, 6);
            int8_t n[3];
            double nn[3] = {raw.nrm[i].x, raw.nrm[i].y, raw.nrm[i].z};
            for (int a = 0; a < 3; a++) n[a] = (int8_t)std::lround(std::max(-127.0, std::min(127.0, nn[a] * 127.0)));
            std::memcpy(&bm.normals[i * 3], n, 3);
            uint16_t uv[2] = {(uint16_t)std::lround(raw.u[i] / umax * 65535.0),
                              (uint16_t)std::lround(raw.v[i] / umax * 65535.0)};
            std::memcpy(&bm.uvs[i * 4], uv, 4);
        }
        if (nv > 65535) bm.flags |= MESH_INFO_FLAGS_32_BIT_INDICES;
    }

    // Greedy meshletiser over the coherent emission order.
    std::vector<uint32_t> meshlet_vertices;
    std::vector<int32_t> stamp(nv, -1);
    std::vector<uint8_t> local(nv, 0);
    size_t ntri = raw.tris.size() / 3;
    size_t t = 0;
    while (t < ntri) {
        Meshlet ml;
        std::memset(&ml, 0, sizeof(ml));
        int32_t id = (int32_t)bm.meshlets.size();
        uint32_t vcount = 0, tcount = 0;
        ml.index_offset = (uint32_t)meshlet_vertices.size();
        ml.triangle_offset = (uint32_t)bm.micro.size();
        while (t < ntri && tcount < MAX_MESHLET_TRIANGLES) {
            uint32_t nnew = 0;
            for (int k = 0; k < 3; k++) {
                uint32_t v = raw.tris[t * 3 + k];
                bool seen = stamp[v] == id;
                for (int q = 0; q < k && !seen; q++) seen = raw.tris[t * 3 + q] == v;
                if (!seen) nnew++;
            }
            if (vcount + nnew > MAX_MESHLET_UNIQUE_VERTICES) break;
            for (int k = 0; k < 3; k++) {
                uint32_t v = raw.tris[t * 3 + k];
                if (stamp[v] != id) {
                    stamp[v] = id;
                    local[v] = (uint8_t)vcount++;
                    meshlet_vertices.push_back(v);
                }
                bm.micro.push_back(local[v]);
            }
            tcount++;
            t++;
        }
        while (bm.micro.size() & 3) bm.micro.push_back(0);  // 4-byte aligned offsets
        ml.triangle_count = (uint8_t)tcount;
        ml.index_count = (uint8_t)vcount;

        // bounding sphere of the meshlet's vertices
        std::vector<const float*> pts;
        for (uint32_t i = 0; i < vcount; i++) pts.push_back(&sp[meshlet_vertices[ml.index_offset + i] * 3]);
        float bs[4];
        ritter_sphere(pts, bs);
        ml.bounding_sphere = {bs[0], bs[1], bs[2], bs[3]};

        // Normal cone.  Axis = mean of unit triangle normals; half angle from
        // the least aligned normal; apex pushed back along the axis until it
        // lies behind every triangle plane, so that the reference's test
        // dot(normalize(apex - eye), axis) >= cutoff (src/shaders/common/
        // culling.glsl:137-151) only rejects meshlets whose triangles all face
        // away from the eye.
        V3 c{bs[0], bs[1], bs[2]};
        std::vector<V3> tn;
        std::vector<V3> tp;
        V3 acc{0, 0, 0};
        for (uint32_t k = 0; k < tcount; k++) {
            const uint8_t* mi = &bm.micro[ml.triangle_offset + k * 3];
            const float* a = &sp[meshlet_vertices[ml.index_offset + mi[0]] * 3];
            const float* b = &sp[meshlet_vertices[ml.index_offset + mi[1]] * 3];
            const float* d = &sp[meshlet_vertices[ml.index_offset + mi[2]] * 3];
            V3 A{a[0], a[1], a[2]}, B{b[0], b[1], b[2]}, D{d[0], d[1], d[2]};
            V3 n = cross(B - A, D - A);
            if (len(n) <= 0) continue;
            n = norm(n);
            tn.push_back(n);
            tp.push_back(A);
            acc = acc + n;
        }
        V3 axis = norm(acc);
        double mindp = 1;
        for (auto& n : tn) mindp = std::min(mindp, dot(axis, n));
        if (tn.empty() || len(axis) == 0 || mindp <= 0.1) {
            ml.cone_apex = {bs[0], bs[1], bs[2]};
            ml.cone_axis = {0, 1, 0};
            ml.cone_cutoff = 2.0f;  // never culls
        } else {
            double tback = 0;
            for (size_t k = 0; k < tn.size(); k++) {
                double need = -dot(tp[k] - c, tn[k]) / dot(axis, tn[k]);
                tback = std::max(tback, need);
            }
            tback = tback * 1.001 + 1e-6 * (double)bs[3];
            V3 apex = c - axis * tback;
            double cutoff = std::sqrt(std::max(0.0, 1 - mindp * mindp)) + 1e-3;
            ml.cone_apex = {(float)apex.x, (float)apex.y, (float)apex.z};
            ml.cone_axis = {(float)axis.x, (float)axis.y, (float)axis.z};
            ml.cone_cutoff = (float)std::min(2.0, cutoff);
        }
        bm.meshlets.push_back(ml);
    }
    // index buffer: the meshlets' vertex lists
    if (bm.flags & MESH_INFO_FLAGS_32_BIT_INDICES) {
        bm.indices.resize(meshlet_vertices.size() * 4);
        std::memcpy(bm.indices.data(), meshlet_vertices.data(), bm.indices.size());
    } else {
        bm.indices.resize(meshlet_vertices.size() * 2);
        for (size_t i = 0; i < meshlet_vertices.size(); i++) {
            uint16_t v = (uint16_t)meshlet_vertices[i];
            std::memcpy(&bm.indices[i * 2], &v, 2);
        }
    }
    while (bm.micro.size() < 16) bm.micro.push_back(0);
    std::vector<const float*> all;
    for (size_t i = 0; i < nv; i++) all.push_back(&sp[i * 3]);
    ritter_sphere(all, bm.bounding_sphere);
    return bm;
}

// ---------------------------------------------------------------- scene
struct Material {
    uint16_t base_tex, mr_tex, normal_tex;
    float factor[3];
    bool alpha_clip;
};

struct TextureData {
    uint32_t w, h, srgb;
    std::vector<uint8_t> texels;
};

struct DeviceAlloc {
    void* ptr = nullptr;
    ~DeviceAlloc() { if (ptr) cudaFree(ptr); }
};

}  // namespace

struct lh_scene {
    uint32_t config_id = 0;
    uint64_t seed = 0;
    uint32_t width = 0, height = 0, shadow_size = 1024;
    std::vector<BuiltMesh> meshes;
    std::vector<Material> materials;
    std::vector<TextureData> textures;
    // per mesh-material combination a MeshInfo (host addresses)
    std::vector<MeshInfo> host_infos;
    std::vector<uint32_t> info_mesh;  // MeshInfo -> mesh index
    std::vector<Instance> host_instances;
    std::vector<uint32_t> instance_info;  // Instance -> MeshInfo index
    std::vector<lh_texture> host_textures;
    // device copy
    int device = -1;
    std::vector<std::unique_ptr<DeviceAlloc>> allocs;
    Instance* device_instances = nullptr;
    std::vector<lh_texture> device_textures;
    std::vector<MeshInfo> device_infos;
    uint64_t device_info_base = 0;
    uint64_t device_bytes = 0;
    Uniforms uniforms;
    std::vector<Uniforms> probes;
    uint64_t total_meshlets = 0, total_triangles = 0;
};

namespace {

static void make_instance(Instance& inst, const M4& model, bool reference_normal_transform) {
    inst.transform = to_f(model);
    M4 inv = inverse(model);
    // normal_transform: inverse-transpose of the upper 3x3 (correct for any
    // rotation), or the reference constructor's mat3(inverse(M))
    // (src/shared_cpu_gpu.h:92-97) when asked.
    for (int c = 0; c < 3; c++) {
        double col[3];
        for (int r = 0; r < 3; r++) col[r] = reference_normal_transform ? inv.m[c][r] : inv.m[r][c];
        inst.normal_transform.cols[c] = {(float)col[0], (float)col[1], (float)col[2]};
    }
}

static M4 trs(V3 t, double yaw, double scale) {
    M4 r = identity();
    double c = std::cos(yaw), s = std::sin(yaw);
    r.m[0][0] = c * scale; r.m[0][2] = -s * scale;
    r.m[1][1] = scale;
    r.m[2][0] = s * scale; r.m[2][2] = c * scale;
    r.m[3][0] = t.x; r.m[3][1] = t.y; r.m[3][2] = t.z;
    return r;
}

static TextureData noise_texture(uint32_t size, uint32_t seed, const double base[3], const double var[3], bool srgb,
                                 bool alpha_holes) {
    TextureData t;
    t.w = t.h = size;
    t.srgb = srgb ? 1 : 0;
    t.texels.resize((size_t)size * size * 4);
    for (uint32_t y = 0; y < size; y++)
        for (uint32_t x = 0; x < size; x++) {
            double n = 0.5 * noise2p(x / 32.0, y / 32.0, (int)(size / 32), seed) +
                       0.3 * noise2p(x / 8.0, y / 8.0, (int)(size / 8), seed + 7) +
                       0.2 * noise2p(x / 2.0, y / 2.0, (int)(size / 2), seed + 13);
            uint8_t* p = &t.texels[((size_t)y * size + x) * 4];
            for (int c = 0; c < 3; c++) p[c] = (uint8_t)std::lround(255.0 * std::min(1.0, std::max(0.0, base[c] + var[c] * (n - 0.5))));
            p[3] = alpha_holes ? (n > 0.55 ? 0 : 255) : 255;
        }
    return t;
}

static TextureData constant_texture(double r, double g, double b, bool srgb) {
    TextureData t;
    t.w = t.h = 1;
    t.srgb = srgb ? 1 : 0;
    t.texels = {(uint8_t)std::lround(r * 255), (uint8_t)std::lround(g * 255), (uint8_t)std::lround(b * 255), 255};
    return t;
}

static void camera_uniforms(lh_scene* s, V3 pos, double yaw, double pitch, double fov, uint32_t w, uint32_t h,
                            Uniforms* out) {
    lh_camera cam;
    std::memset(&cam, 0, sizeof(cam));
    cam.position = {(float)pos.x, (float)pos.y, (float)pos.z};
    cam.yaw = (float)yaw;
    cam.pitch = (float)pitch;
    cam.fov_degrees = (float)fov;
    cam.sun_latitude = -5.6f;  // src/main.cpp:611-612
    cam.sun_longitude = 1.37f;
    cam.width = w;
    cam.height = h;
    cam.shadow_cam_distance = 1024.0f;  // src/main.cpp:653-654
    cam.cascade_split_pow = 3.0f;
    cam.num_instances = (uint32_t)s->host_instances.size();
    lh_make_uniforms(&cam, out);
}

static void finish_infos(lh_scene* s) {
    for (size_t i = 0; i < s->host_infos.size(); i++) {
        MeshInfo& mi = s->host_infos[i];
        const BuiltMesh& m = s->meshes[s->info_mesh[i]];
        mi.positions = (uint64_t)(uintptr_t)m.positions.data();
        mi.indices = (uint64_t)(uintptr_t)m.indices.data();
        mi.normals = (uint64_t)(uintptr_t)m.normals.data();
        mi.uvs = (uint64_t)(uintptr_t)m.uvs.data();
        mi.micro_indices = (uint64_t)(uintptr_t)m.micro.data();
        mi.meshlets = (uint64_t)(uintptr_t)m.meshlets.data();
    }
    for (size_t i = 0; i < s->host_instances.size(); i++)
        s->host_instances[i].mesh_info_address = (uint64_t)(uintptr_t)&s->host_infos[s->instance_info[i]];
    s->host_textures.clear();
    for (auto& t : s->textures) {
        lh_texture d;
        d.texels = (uint64_t)(uintptr_t)t.texels.data();
        d.width = t.w;
        d.height = t.h;
        d.srgb = t.srgb;
        d.reserved = 0;
        s->host_textures.push_back(d);
    }
    s->total_meshlets = 0;
    s->total_triangles = 0;
    for (size_t i = 0; i < s->host_instances.size(); i++) {
        const BuiltMesh& m = s->meshes[s->info_mesh[s->instance_info[i]]];
        s->total_meshlets += m.meshlets.size();
        s->total_triangles += m.n_triangles;
    }
}

// One MeshInfo per (mesh, material) pair actually used.
static uint32_t info_for(lh_scene* s, uint32_t mesh, uint32_t mat, std::vector<int64_t>& cache) {
    size_t key = (size_t)mesh * s->materials.size() + mat;
    if (cache[key] >= 0) return (uint32_t)cache[key];
    const BuiltMesh& m = s->meshes[mesh];
    const Material& mt = s->materials[mat];
    MeshInfo mi;
    std::memset(&mi, 0, sizeof(mi));
    mi.num_meshlets = (uint16_t)m.meshlets.size();
    mi.flags = (uint8_t)(m.flags | (mt.alpha_clip ? MESH_INFO_FLAGS_ALPHA_CLIP : 0));
    mi.bounding_sphere = {m.bounding_sphere[0], m.bounding_sphere[1], m.bounding_sphere[2], m.bounding_sphere[3]};
    mi.texture_scale = {m.tex_scale[0], m.tex_scale[1]};
    mi.texture_offset = {0, 0};
    mi.base_color_texture_index = mt.base_tex;
    mi.metallic_roughness_texture_index = mt.mr_tex;
    mi.normal_texture_index = mt.normal_tex;
    mi.base_color_factor = {mt.factor[0], mt.factor[1], mt.factor[2]};
    s->host_infos.push_back(mi);
    s->info_mesh.push_back(mesh);
    cache[key] = (int64_t)s->host_infos.size() - 1;
    return (uint32_t)cache[key];
}

static void add_materials(lh_scene* s, Rng& rng, uint32_t n, bool textured, bool alpha_odd) {
    for (uint32_t i = 0; i < n; i++) {
        double base[3] = {rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9)};
        double var[3] = {0.4, 0.4, 0.4};
        bool alpha = alpha_odd && (i & 1);
        uint16_t bt = (uint16_t)s->textures.size();
        if (textured)
            s->textures.push_back(noise_texture(256, (uint32_t)rng.next(), base, var, true, alpha));
        else
            s->textures.push_back(constant_texture(base[0], base[1], base[2], true));
        uint16_t mr = (uint16_t)s->textures.size();
        double rough = rng.uniform(0.25, 0.9), metal = rng.uniform() < 0.25 ? rng.uniform(0.5, 1.0) : 0.0;
        s->textures.push_back(constant_texture(1.0, rough, metal, false));
        Material m;
        m.base_tex = bt;
        m.mr_tex = mr;
        m.normal_tex = (uint16_t)UNUSED_TEXTURE_INDEX;
        m.factor[0] = (float)rng.uniform(0.8, 1.0);
        m.factor[1] = (float)rng.uniform(0.8, 1.0);
        m.factor[2] = (float)rng.uniform(0.8, 1.0);
        m.alpha_clip = alpha;
        s->materials.push_back(m);
    }
}

static int grid_n(double tris) { return std::max(2, (int)std::lround(std::sqrt(tris / 12.0))); }

static void build_config(lh_scene* s, uint32_t cfg, const lh_scene_params& p) {
    Rng rng(s->seed);
    double detail = p.detail > 0 ? p.detail : 1.0;
    bool q = p.quantized != 0;
    bool refnt = p.reference_normal_transform != 0;
    std::vector<int64_t> cache;
    auto reset_cache = [&]() { cache.assign(s->meshes.size() * s->materials.size(), -1); };

    if (cfg == 1) {
        // 64 icospheres of 20,480 triangles, uniform in a 200 m cube.
        s->width = p.width ? p.width : 1280;
        s->height = p.height ? p.height : 720;
        int levels = 5;
        if (detail < 0.2) levels = 3; else if (detail < 0.6) levels = 4;
        s->meshes.push_back(build_mesh(icosphere(levels), q));
        add_materials(s, rng, 4, false, p.alpha_clip_materials != 0);
        reset_cache();
        uint32_t n = p.n_instances ? p.n_instances : 64;
        for (uint32_t i = 0; i < n; i++) {
            V3 t{rng.uniform(-100, 100), rng.uniform(-100, 100), rng.uniform(-100, 100)};
            double yaw = rng.uniform(0, 6.283185307179586), sc = rng.uniform(0.5, 2.0);
            uint32_t mat = (uint32_t)(rng.next() % s->materials.size());
            Instance inst;
            std::memset(&inst, 0, sizeof(inst));
            make_instance(inst, mul(trs(t, yaw, sc), s->meshes[0].dequant), refnt);
            s->host_instances.push_back(inst);
            s->instance_info.push_back(info_for(s, 0, mat, cache));
        }
        camera_uniforms(s, V3{0, 0, -150}, 1.5707963267948966, 0.0, 60.0, s->width, s->height, &s->uniforms);
        return;
    }

    // Configs 2-5: clustered placement of several procedural meshes.
    struct MeshSpec { int kind; double tris; uint32_t count; double size; };
    std::vector<MeshSpec> specs;
    uint32_t n_inst;
    double area = 1000.0;
    uint32_t n_mat = 16;
    if (cfg == 4) {
        s->width = p.width ? p.width : 512;
        s->height = p.height ? p.height : 512;
        specs = {{0, 5000, 800, 2.0}, {1, 12000, 600, 2.5}, {2, 25000, 400, 2.0}, {0, 50000, 248, 3.0}};
        n_inst = 2048;
        area = 400.0;
        n_mat = 8;
    } else if (cfg == 5) {
        s->width = p.width ? p.width : 3840;
        s->height = p.height ? p.height : 2160;
        specs = {{0, 10000, 20000, 2.0}, {1, 12000, 15000, 2.5}, {2, 14000, 15000, 2.0}, {0, 20000, 12000, 2.5},
                 {1, 30000, 10000, 3.0}, {2, 40000, 8000, 3.0}, {0, 60000, 6000, 3.5}, {1, 80000, 4000, 3.5},
                 {2, 100000, 3000, 4.0}, {0, 150000, 2000, 4.0}, {1, 200000, 1500, 5.0}, {3, 20000, 1500, 3.0},
                 {2, 250000, 1000, 5.0}, {0, 300000, 500, 6.0}, {1, 400000, 300, 6.0}, {0, 500000, 200, 8.0}};
        n_inst = 100000;
        area = 2000.0;
    } else {
        s->width = p.width ? p.width : 1920;
        s->height = p.height ? p.height : 1080;
        specs = {{0, 10000, 1500, 2.0}, {1, 10000, 1250, 2.5}, {2, 12000, 600, 2.0}, {0, 12000, 400, 3.0},
                 {1, 16000, 200, 3.0}, {2, 40000, 90, 4.0}, {0, 100000, 36, 5.0}, {1, 200000, 20, 6.0}};
        n_inst = 4096;
    }
    if (cfg == 3) s->shadow_size = 2048;
    if (p.n_instances) n_inst = p.n_instances;

    uint32_t mesh_seed = (uint32_t)rng.next();
    for (size_t k = 0; k < specs.size(); k++) {
        double tris = specs[k].tris * detail;
        RawMesh raw;
        switch (specs[k].kind) {
            case 0: raw = cube_mesh(grid_n(tris), true, 0.35, mesh_seed + (uint32_t)k, V3{1, 1, 1}); break;
            case 1: {
                int nv = std::max(3, (int)std::lround(std::sqrt(tris / 2.0 / 3.0)));
                raw = torus(nv * 3, nv, 1.0, 0.35);
                break;
            }
            case 2: raw = cube_mesh(grid_n(tris), false, 0, 0, V3{rng.uniform(0.5, 1.0), rng.uniform(0.5, 1.0), rng.uniform(0.5, 1.0)}); break;
            default: raw = slivers(std::max(8, (int)tris), mesh_seed + (uint32_t)k); break;
        }
        s->meshes.push_back(build_mesh(raw, q));
    }
    add_materials(s, rng, n_mat, true, p.alpha_clip_materials != 0);
    reset_cache();

    // Gaussian mixture of 8 clusters over the area.
    struct Cluster { V3 c; double sigma; double w; };
    std::vector<Cluster> clusters;
    double wsum = 0;
    for (int k = 0; k < 8; k++) {
        Cluster c;
        c.c = V3{rng.uniform(-area * 0.4, area * 0.4), 0, rng.uniform(-area * 0.4, area * 0.4)};
        c.sigma = rng.uniform(30, 80) * area / 1000.0;
        c.w = k == 0 ? 3.0 : rng.uniform(0.5, 1.5);
        wsum += c.w;
        clusters.push_back(c);
    }
    // mesh assignment: exact counts per spec, scaled to n_inst
    std::vector<uint32_t> mesh_of;
    uint32_t spec_total = 0;
    for (auto& sp : specs) spec_total += sp.count;
    for (size_t k = 0; k < specs.size(); k++) {
        uint32_t c = (uint32_t)std::lround((double)specs[k].count * n_inst / spec_total);
        for (uint32_t i = 0; i < c; i++) mesh_of.push_back((uint32_t)k);
    }
    while (mesh_of.size() < n_inst) mesh_of.push_back(0);
    mesh_of.resize(n_inst);
    for (size_t i = mesh_of.size(); i > 1; i--) std::swap(mesh_of[i - 1], mesh_of[rng.next() % i]);

    for (uint32_t i = 0; i < n_inst; i++) {
        double pick = rng.uniform(0, wsum);
        size_t k = 0;
        while (k + 1 < clusters.size() && pick > clusters[k].w) { pick -= clusters[k].w; k++; }
        V3 t{clusters[k].c.x + rng.normal() * clusters[k].sigma, 0, clusters[k].c.z + rng.normal() * clusters[k].sigma};
        uint32_t mesh = mesh_of[i];
        double sc = specs[mesh].size * rng.uniform(0.5, 1.5);
        t.y = sc * rng.uniform(0.8, 3.0);
        double yaw = rng.uniform(0, 6.283185307179586);
        uint32_t mat = (uint32_t)(rng.next() % s->materials.size());
        Instance inst;
        std::memset(&inst, 0, sizeof(inst));
        make_instance(inst, mul(trs(t, yaw, sc), s->meshes[mesh].dequant), refnt);
        s->host_instances.push_back(inst);
        s->instance_info.push_back(info_for(s, mesh, mat, cache));
    }
    // Camera inside the heaviest cluster, looking across it.
    V3 cc = clusters[0].c;
    double cam_yaw = rng.uniform(0, 6.283185307179586);
    V3 cam{cc.x - std::cos(cam_yaw) * clusters[0].sigma * 0.5, 6.0, cc.z - std::sin(cam_yaw) * clusters[0].sigma * 0.5};
    double cam_pitch = -0.05;
    if (cfg == 5) {
        // The stress view looks down into the densest cluster from 60 m: the
        // visible meshlets must fit the 24-bit draw slot of the visibility ID
        // (util.glsl:18-20), and the view stays deep (depth complexity ~10).
        cam.y = 60.0;
        cam_pitch = -0.8;
    }
    camera_uniforms(s, cam, cam_yaw, cam_pitch, 60.0, s->width, s->height, &s->uniforms);

    uint32_t n_probes = p.n_probes ? p.n_probes : (cfg == 3 ? 32 : 0);
    for (uint32_t i = 0; i < n_probes; i++) {
        V3 pos{cc.x + rng.normal() * clusters[0].sigma * 0.5, rng.uniform(2, 20), cc.z + rng.normal() * clusters[0].sigma * 0.5};
        uint32_t w = (uint32_t)std::lround(std::exp(rng.uniform(std::log(64.0), std::log(512.0))));
        uint32_t h = (uint32_t)std::lround(std::exp(rng.uniform(std::log(64.0), std::log(512.0))));
        Uniforms u;
        camera_uniforms(s, pos, rng.uniform(0, 6.283185307179586), rng.uniform(-0.4, 0.2), rng.uniform(50, 90), w, h, &u);
        s->probes.push_back(u);
    }
}

template <class T>
static lh_status upload(lh_scene* s, const T* src, size_t bytes, uint64_t* out) {
    auto a = std::make_unique<DeviceAlloc>();
    size_t sz = bytes ? bytes : 16;
    if (cudaMalloc(&a->ptr, sz) != cudaSuccess) return LH_ERR_OUT_OF_MEMORY;
    if (bytes && cudaMemcpy(a->ptr, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return LH_ERR_CUDA;
    *out = (uint64_t)(uintptr_t)a->ptr;
    s->device_bytes += sz;
    s->allocs.push_back(std::move(a));
    return LH_OK;
}

}  // namespace

namespace {

// ------------------------------------------------------------ scene dumps
constexpr char kDumpMagic[8] = {'L', 'H', 'S', 'C', 'E', 'N', 'E', '\0'};
constexpr uint32_t kDumpVersion = 1;

struct DumpWriter {
    std::vector<uint8_t> out;
    void bytes(const void* p, size_t n) {
        if (n) out.insert(out.end(), static_cast<const uint8_t*>(p), static_cast<const uint8_t*>(p) + n);
    }
    template <class T>
    void pod(const T& v) { bytes(&v, sizeof(T)); }
    void blob(const std::vector<uint8_t>& v) {
        pod((uint64_t)v.size());
        bytes(v.data(), v.size());
    }
};

// Reads from a byte range; the first read past its end clears `ok` and every
// later read then fails too.
struct DumpReader {
    const uint8_t* p;
    size_t left;
    bool ok = true;
    bool bytes(void* dst, size_t n) {
        if (!ok || n > left) return ok = false;
        if (n) std::memcpy(dst, p, n);
        p += n;
        left -= n;
        return true;
    }
    template <class T>
    bool pod(T& v) { return bytes(&v, sizeof(T)); }
    bool blob(std::vector<uint8_t>& v) {
        uint64_t n = 0;
        if (!pod(n) || n > left) return ok = false;
        v.resize((size_t)n);
        return bytes(v.data(), (size_t)n);
    }
    template <class T>
    bool array(std::vector<T>& v, uint64_t n) {
        if (!ok || n > left / sizeof(T)) return ok = false;
        v.resize((size_t)n);
        return bytes(v.data(), (size_t)n * sizeof(T));
    }
};

// Every read a mesh's meshlets lead to stays inside its buffers: attribute
// buffers hold n_vertices entries in the mesh's format, every index names a
// vertex, every meshlet's index and micro-index ranges lie in their arrays
// and its micro-indices name its own vertices.
static bool dump_mesh_consistent(const BuiltMesh& m) {
    const bool fp32 = (m.flags & MESH_INFO_FLAGS_FP32_VERTICES) != 0;
    const bool idx32 = (m.flags & MESH_INFO_FLAGS_32_BIT_INDICES) != 0;
    const uint64_t nv = m.n_vertices;
    if (m.positions.size() < nv * (fp32 ? 12u : 6u) || m.normals.size() < nv * (fp32 ? 12u : 3u) ||
        m.uvs.size() < nv * (fp32 ? 8u : 4u))
        return false;
    const size_t isz = idx32 ? 4u : 2u;
    if (m.indices.size() % isz != 0 || m.meshlets.size() > 0xFFFFu) return false;
    const size_t n_idx = m.indices.size() / isz;
    for (size_t i = 0; i < n_idx; i++) {
        uint32_t v = 0;
        if (idx32) {
            std::memcpy(&v, &m.indices[i * 4], 4);
        } else {
            uint16_t h;
            std::memcpy(&h, &m.indices[i * 2], 2);
            v = h;
        }
        if (v >= nv) return false;
    }
    for (const Meshlet& ml : m.meshlets) {
        if ((uint64_t)ml.index_offset + ml.index_count > n_idx) return false;
        if ((uint64_t)ml.triangle_offset + 3u * ml.triangle_count > m.micro.size()) return false;
        for (uint32_t k = 0; k < 3u * ml.triangle_count; k++)
            if (m.micro[ml.triangle_offset + k] >= ml.index_count) return false;
    }
    return true;
}

}  // namespace

extern "C" {

lh_status lh_make_uniforms(const lh_camera* c, Uniforms* out) {
    if (!c || !out || c->width == 0 || c->height == 0) return LH_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    // CameraParams::facing / sun_dir (src/input.h:31-49), in float.
    float yaw = c->yaw, pitch = c->pitch;
    V3 facing{std::cos(yaw) * std::cos(pitch), std::sin(pitch), std::sin(yaw) * std::cos(pitch)};
    V3 pos{c->position.x, c->position.y, c->position.z};
    M4 view = look_at(pos, pos + facing, V3{0, 1, 0});
    view = from_f(to_f(view));  // the reference keeps float matrices
    M4 persp = infinite_reverse_z_perspective(c->fov_degrees * 3.14159265358979323846f / 180.0f, (float)c->width,
                                              (float)c->height, NEAR_PLANE);
    M4 pv = from_f(to_f(mul(persp, view)));
    out->combined_perspective_view = to_f(pv);
    out->inv_perspective_view = to_f(inverse(pv));
    out->view = to_f(view);
    out->initial_view = to_f(view);
    out->perspective = to_f(persp);
    out->perspective_inverse = to_f(inverse(persp));
    out->view_inverse = to_f(inverse(view));
    out->camera_pos = c->position;
    float sl = c->sun_latitude, so = c->sun_longitude;
    out->sun_dir = {std::cos(sl) * std::cos(so), std::sin(so), std::sin(sl) * std::cos(so)};
    out->sun_intensity = {1.0f, 1.0f, 1.0f};
    out->num_instances = c->num_instances;
    out->window_size = {c->width, c->height};
    out->shadow_cam_distance = c->shadow_cam_distance;
    out->cascade_split_pow = c->cascade_split_pow;
    out->debug = UNIFORMS_DEBUG_OFF;
    out->debug_shadowmaps = 0;
    return LH_OK;
}

lh_status lh_scene_create(uint32_t config_id, uint64_t seed, const lh_scene_params* params, lh_scene** out) {
    if (!out || config_id < 1 || config_id > 5) return LH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    lh_scene_params p;
    std::memset(&p, 0, sizeof(p));
    if (params) p = *params;
    lh_scene* s = new (std::nothrow) lh_scene();
    if (!s) return LH_ERR_OUT_OF_MEMORY;
    s->config_id = config_id;
    s->seed = seed;
    try {
        build_config(s, config_id, p);
    } catch (...) {
        delete s;
        return LH_ERR_OUT_OF_MEMORY;
    }
    for (auto& m : s->meshes)
        if (m.meshlets.size() > 65535) { delete s; return LH_ERR_CAPACITY; }  // num_meshlets is u16
    finish_infos(s);
    *out = s;
    return LH_OK;
}

lh_status lh_scene_from_mesh(const float* positions, const float* normals, const float* uvs, uint32_t n_vertices,
                             const uint32_t* indices, uint32_t n_triangles, const lh_mat4* transforms,
                             uint32_t n_instances, const Uniforms* uniforms, lh_scene** out) {
    if (!out || !positions || !indices || !transforms || !uniforms || n_vertices == 0 || n_triangles == 0 ||
        n_instances == 0 || uniforms->window_size.x == 0 || uniforms->window_size.y == 0)
        return LH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    for (uint64_t i = 0; i < (uint64_t)n_triangles * 3; i++)
        if (indices[i] >= n_vertices) return LH_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < (uint64_t)n_vertices * 3; i++)
        if (!std::isfinite(positions[i])) return LH_ERR_INVALID_ARGUMENT;
    lh_scene* s = new (std::nothrow) lh_scene();
    if (!s) return LH_ERR_OUT_OF_MEMORY;
    try {
        RawMesh raw;
        raw.pos.resize(n_vertices);
        raw.u.assign(n_vertices, 0.0);
        raw.v.assign(n_vertices, 0.0);
        for (uint32_t i = 0; i < n_vertices; i++) {
            raw.pos[i] = V3{positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]};
            if (uvs) {
                raw.u[i] = uvs[2 * i];
                raw.v[i] = uvs[2 * i + 1];
            }
        }
        raw.tris.assign(indices, indices + (size_t)n_triangles * 3);
        if (normals) {
            raw.nrm.resize(n_vertices);
            for (uint32_t i = 0; i < n_vertices; i++) {
                V3 n = norm(V3{normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]});
                raw.nrm[i] = len(n) > 0 ? n : V3{0, 1, 0};
            }
        } else {
            compute_vertex_normals(raw);
        }
        s->config_id = 0;
        s->seed = 0;
        s->width = uniforms->window_size.x;
        s->height = uniforms->window_size.y;
        s->meshes.push_back(build_mesh(raw, false));
        if (s->meshes[0].meshlets.size() > 65535) {
            delete s;
            return LH_ERR_CAPACITY;  // num_meshlets is u16
        }
        // one untextured material: light grey base colour, roughness 0.5
        s->textures.push_back(constant_texture(0.8, 0.8, 0.8, true));
        s->textures.push_back(constant_texture(1.0, 0.5, 0.0, false));
        Material m;
        m.base_tex = 0;
        m.mr_tex = 1;
        m.normal_tex = (uint16_t)UNUSED_TEXTURE_INDEX;
        m.factor[0] = m.factor[1] = m.factor[2] = 1.0f;
        m.alpha_clip = false;
        s->materials.push_back(m);
        std::vector<int64_t> cache(1, -1);
        const uint32_t info = info_for(s, 0, 0, cache);
        for (uint32_t i = 0; i < n_instances; i++) {
            Instance inst;
            std::memset(&inst, 0, sizeof(inst));
            make_instance(inst, mul(from_f(transforms[i]), s->meshes[0].dequant), false);
            s->host_instances.push_back(inst);
            s->instance_info.push_back(info);
        }
        s->uniforms = *uniforms;
        s->uniforms.num_instances = n_instances;
    } catch (...) {
        delete s;
        return LH_ERR_OUT_OF_MEMORY;
    }
    finish_infos(s);
    *out = s;
    return LH_OK;
}

lh_status lh_scene_describe(const lh_scene* s, lh_scene_desc* d) {
    if (!s || !d) return LH_ERR_INVALID_ARGUMENT;
    std::memset(d, 0, sizeof(*d));
    d->config_id = s->config_id;
    d->n_instances = (uint32_t)s->host_instances.size();
    d->n_meshes = (uint32_t)s->meshes.size();
    d->n_textures = (uint32_t)s->textures.size();
    d->n_probes = (uint32_t)s->probes.size();
    d->width = s->width;
    d->height = s->height;
    d->shadow_size = s->shadow_size;
    d->total_meshlets = s->total_meshlets;
    d->total_triangles = s->total_triangles;
    d->seed = s->seed;
    d->host_instances = s->host_instances.data();
    d->host_textures = s->host_textures.data();
    d->device_instances = s->device_instances;
    d->device_textures = s->device_textures.empty() ? nullptr : s->device_textures.data();
    d->uniforms = s->uniforms;
    d->probes = s->probes.empty() ? nullptr : s->probes.data();
    d->device_bytes = s->device_bytes;
    return LH_OK;
}

lh_status lh_scene_upload(lh_scene* s, int device) {
    if (!s) return LH_ERR_INVALID_ARGUMENT;
    if (s->device_instances) return LH_OK;
    if (cudaSetDevice(device) != cudaSuccess) return LH_ERR_CUDA;
    s->device = device;
    std::vector<MeshInfo> dinfos = s->host_infos;
    std::vector<uint64_t> dpos(s->meshes.size()), didx(s->meshes.size()), dnrm(s->meshes.size()),
        duv(s->meshes.size()), dmicro(s->meshes.size()), dml(s->meshes.size());
    for (size_t m = 0; m < s->meshes.size(); m++) {
        const BuiltMesh& bm = s->meshes[m];
        lh_status st;
        if ((st = upload(s, bm.positions.data(), bm.positions.size(), &dpos[m])) != LH_OK) return st;
        if ((st = upload(s, bm.indices.data(), bm.indices.size(), &didx[m])) != LH_OK) return st;
        if ((st = upload(s, bm.normals.data(), bm.normals.size(), &dnrm[m])) != LH_OK) return st;
        if ((st = upload(s, bm.uvs.data(), bm.uvs.size(), &duv[m])) != LH_OK) return st;
        if ((st = upload(s, bm.micro.data(), bm.micro.size(), &dmicro[m])) != LH_OK) return st;
        if ((st = upload(s, bm.meshlets.data(), bm.meshlets.size() * sizeof(Meshlet), &dml[m])) != LH_OK) return st;
    }
    for (size_t i = 0; i < dinfos.size(); i++) {
        uint32_t m = s->info_mesh[i];
        dinfos[i].positions = dpos[m];
        dinfos[i].indices = didx[m];
        dinfos[i].normals = dnrm[m];
        dinfos[i].uvs = duv[m];
        dinfos[i].micro_indices = dmicro[m];
        dinfos[i].meshlets = dml[m];
    }
    uint64_t dinfo_base;
    lh_status st;
    if ((st = upload(s, dinfos.data(), dinfos.size() * sizeof(MeshInfo), &dinfo_base)) != LH_OK) return st;
    s->device_infos = dinfos;
    s->device_info_base = dinfo_base;
    std::vector<Instance> dinst = s->host_instances;
    for (size_t i = 0; i < dinst.size(); i++) dinst[i].mesh_info_address = dinfo_base + s->instance_info[i] * sizeof(MeshInfo);
    uint64_t dinst_ptr;
    if ((st = upload(s, dinst.data(), dinst.size() * sizeof(Instance), &dinst_ptr)) != LH_OK) return st;
    s->device_textures.clear();
    for (auto& t : s->textures) {
        uint64_t p;
        if ((st = upload(s, t.texels.data(), t.texels.size(), &p)) != LH_OK) return st;
        lh_texture d;
        d.texels = p;
        d.width = t.w;
        d.height = t.h;
        d.srgb = t.srgb;
        d.reserved = 0;
        s->device_textures.push_back(d);
    }
    s->device_instances = (Instance*)(uintptr_t)dinst_ptr;
    return LH_OK;
}

uint32_t lh_scene_mesh_count(const lh_scene* s) { return s ? (uint32_t)s->host_infos.size() : 0; }

lh_status lh_scene_mesh_get(const lh_scene* s, uint32_t i, lh_scene_mesh* out) {
    if (!s || !out || i >= s->host_infos.size()) return LH_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->host_info = &s->host_infos[i];
    const BuiltMesh& m = s->meshes[s->info_mesh[i]];
    out->mesh = s->info_mesh[i];
    out->vertices = m.n_vertices;
    out->triangles = m.n_triangles;
    out->flags = s->host_infos[i].flags;
    if (!s->device_infos.empty()) {
        out->device_info = s->device_info_base + (uint64_t)i * sizeof(MeshInfo);
        out->device_positions = s->device_infos[i].positions;
        out->device_normals = s->device_infos[i].normals;
        out->device_uvs = s->device_infos[i].uvs;
    }
    return LH_OK;
}

lh_status lh_scene_instance_records(const lh_scene* s, uint32_t* out) {
    if (!s || !out) return LH_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < s->instance_info.size(); i++) out[i] = s->instance_info[i];
    return LH_OK;
}

lh_status lh_scene_save(const lh_scene* s, const char* path) {
    if (!s || !path) return LH_ERR_INVALID_ARGUMENT;
    DumpWriter w;
    w.bytes(kDumpMagic, sizeof(kDumpMagic));
    w.pod(kDumpVersion);
    w.pod((uint32_t)0);
    w.pod(s->config_id);
    w.pod(s->width);
    w.pod(s->height);
    w.pod(s->shadow_size);
    w.pod(s->seed);
    w.pod(s->uniforms);
    w.pod((uint32_t)s->probes.size());
    for (const Uniforms& u : s->probes) w.pod(u);
    w.pod((uint32_t)s->meshes.size());
    for (const BuiltMesh& m : s->meshes) {
        w.pod(m.flags);
        w.pod(m.n_vertices);
        w.pod(m.n_triangles);
        w.bytes(m.bounding_sphere, sizeof(m.bounding_sphere));
        w.bytes(m.tex_scale, sizeof(m.tex_scale));
        w.bytes(m.dequant.m, sizeof(m.dequant.m));
        w.blob(m.positions);
        w.blob(m.normals);
        w.blob(m.uvs);
        w.blob(m.indices);
        w.blob(m.micro);
        w.pod((uint64_t)m.meshlets.size());
        w.bytes(m.meshlets.data(), m.meshlets.size() * sizeof(Meshlet));
    }
    w.pod((uint32_t)s->host_infos.size());
    for (size_t i = 0; i < s->host_infos.size(); i++) {
        MeshInfo mi = s->host_infos[i];
        mi.positions = mi.indices = mi.normals = mi.uvs = mi.micro_indices = mi.meshlets = 0;
        w.pod(mi);
        w.pod(s->info_mesh[i]);
    }
    w.pod((uint32_t)s->textures.size());
    for (const TextureData& t : s->textures) {
        w.pod(t.w);
        w.pod(t.h);
        w.pod(t.srgb);
        w.blob(t.texels);
    }
    w.pod((uint32_t)s->host_instances.size());
    for (size_t i = 0; i < s->host_instances.size(); i++) {
        Instance inst = s->host_instances[i];
        inst.mesh_info_address = 0;
        w.pod(inst);
        w.pod(s->instance_info[i]);
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return LH_ERR_UNSUPPORTED;
    const bool wrote = std::fwrite(w.out.data(), 1, w.out.size(), f) == w.out.size();
    return std::fclose(f) == 0 && wrote ? LH_OK : LH_ERR_UNSUPPORTED;
}

lh_status lh_scene_load(const char* path, lh_scene** out) {
    if (!path || !out) return LH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::vector<uint8_t> file;
    {
        FILE* f = std::fopen(path, "rb");
        if (!f) return LH_ERR_UNSUPPORTED;
        uint8_t chunk[1 << 16];
        size_t n;
        while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) file.insert(file.end(), chunk, chunk + n);
        const bool failed = std::ferror(f) != 0;
        std::fclose(f);
        if (failed) return LH_ERR_UNSUPPORTED;
    }
    DumpReader r{file.data(), file.size()};
    char magic[sizeof(kDumpMagic)];
    uint32_t version = 0, reserved = 0;
    if (!r.bytes(magic, sizeof(magic)) || std::memcmp(magic, kDumpMagic, sizeof(magic)) != 0 || !r.pod(version) ||
        version != kDumpVersion || !r.pod(reserved))
        return LH_ERR_INVALID_ARGUMENT;
    std::unique_ptr<lh_scene> s(new (std::nothrow) lh_scene());
    if (!s) return LH_ERR_OUT_OF_MEMORY;
    uint32_t n_probes = 0, n_meshes = 0, n_infos = 0, n_textures = 0, n_instances = 0;
    r.pod(s->config_id);
    r.pod(s->width);
    r.pod(s->height);
    r.pod(s->shadow_size);
    r.pod(s->seed);
    r.pod(s->uniforms);
    r.pod(n_probes);
    r.array(s->probes, n_probes);
    r.pod(n_meshes);
    if (!r.ok || n_meshes > r.left) return LH_ERR_INVALID_ARGUMENT;
    s->meshes.resize(n_meshes);
    for (BuiltMesh& m : s->meshes) {
        uint64_t n_meshlets = 0;
        r.pod(m.flags);
        r.pod(m.n_vertices);
        r.pod(m.n_triangles);
        r.bytes(m.bounding_sphere, sizeof(m.bounding_sphere));
        r.bytes(m.tex_scale, sizeof(m.tex_scale));
        r.bytes(m.dequant.m, sizeof(m.dequant.m));
        r.blob(m.positions);
        r.blob(m.normals);
        r.blob(m.uvs);
        r.blob(m.indices);
        r.blob(m.micro);
        r.pod(n_meshlets);
        r.array(m.meshlets, n_meshlets);
        if (!r.ok || !dump_mesh_consistent(m)) return LH_ERR_INVALID_ARGUMENT;
    }
    r.pod(n_infos);
    if (!r.ok || n_infos > r.left / (sizeof(MeshInfo) + 4)) return LH_ERR_INVALID_ARGUMENT;
    s->host_infos.resize(n_infos);
    s->info_mesh.resize(n_infos);
    for (uint32_t i = 0; i < n_infos; i++) {
        r.pod(s->host_infos[i]);
        r.pod(s->info_mesh[i]);
        if (!r.ok || s->info_mesh[i] >= n_meshes ||
            s->host_infos[i].num_meshlets > s->meshes[s->info_mesh[i]].meshlets.size() ||
            (s->host_infos[i].flags & ~MESH_INFO_FLAGS_ALPHA_CLIP) != s->meshes[s->info_mesh[i]].flags)
            return LH_ERR_INVALID_ARGUMENT;
    }
    r.pod(n_textures);
    if (!r.ok || n_textures > r.left) return LH_ERR_INVALID_ARGUMENT;
    s->textures.resize(n_textures);
    for (TextureData& t : s->textures) {
        r.pod(t.w);
        r.pod(t.h);
        r.pod(t.srgb);
        r.blob(t.texels);
        if (!r.ok || t.w == 0 || t.h == 0 || (uint64_t)t.w * t.h * 4 != t.texels.size()) return LH_ERR_INVALID_ARGUMENT;
    }
    r.pod(n_instances);
    if (!r.ok || n_instances > r.left / (sizeof(Instance) + 4)) return LH_ERR_INVALID_ARGUMENT;
    s->host_instances.resize(n_instances);
    s->instance_info.resize(n_instances);
    for (uint32_t i = 0; i < n_instances; i++) {
        r.pod(s->host_instances[i]);
        r.pod(s->instance_info[i]);
        if (!r.ok || s->instance_info[i] >= n_infos) return LH_ERR_INVALID_ARGUMENT;
    }
    if (!r.ok || r.left != 0) return LH_ERR_INVALID_ARGUMENT;
    finish_infos(s.get());
    *out = s.release();
    return LH_OK;
}

void lh_scene_destroy(lh_scene* s) {
    if (!s) return;
    if (s->device >= 0) cudaSetDevice(s->device);
    delete s;
}

}  // extern "C"
