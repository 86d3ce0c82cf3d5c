// Host check of lighthugger_gb300/csrc/sphere_box.cuh: whenever the test
// says a world sphere reaches no pixel centre of a view, points sampled in
// the sphere's box, taken through the raster's own float transform and
// 1/256-pixel snap, must leave a gap without pixel centres on one axis.
// Random perspective (reverse-Z, w = view depth) and orthographic views,
// spheres from 1e-3 to 50 units at distances 0.5 to 3000.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "sphere_box.cuh"

struct ViewFrame {
    float a[3], b[3], c[3], e[3], sx, sy;
};

static lh_mat4 make_view(std::mt19937_64& rng, bool ortho, float& W, float& H, ViewFrame& vf) {
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    // a random rotation (Gram-Schmidt of random vectors) and eye point
    float a[3] = {U(rng), U(rng), U(rng)}, b[3] = {U(rng), U(rng), U(rng)};
    auto norm = [](float* v) {
        const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int i = 0; i < 3; i++) v[i] /= l;
    };
    norm(a);
    const float d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    for (int i = 0; i < 3; i++) b[i] -= d * a[i];
    norm(b);
    float c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const float e[3] = {U(rng) * 500.0f, U(rng) * 500.0f, U(rng) * 500.0f};
    const float sizes[] = {64.0f, 512.0f, 1024.0f, 1920.0f, 2048.0f};
    W = sizes[rng() % 5];
    H = ortho ? W : sizes[rng() % 5];
    // rows of the 4x4: x, y, z, w of the clip position for world p
    float rows[4][4];
    const float sx = ortho ? 2.0f / (10.0f + 500.0f * (U(rng) + 1.0f)) : 1.0f / std::tan(0.4f + 0.4f * (U(rng) + 1.0f));
    const float sy = ortho ? sx : sx * W / H;
    const float* axis[3] = {a, b, c};
    for (int r = 0; r < 3; r++) {
        const float s = r == 0 ? sx : (r == 1 ? sy : 1.0f);
        for (int j = 0; j < 3; j++) rows[r][j] = s * axis[r][j];
        rows[r][3] = -s * (axis[r][0] * e[0] + axis[r][1] * e[1] + axis[r][2] * e[2]);
    }
    if (ortho) {
        rows[3][0] = rows[3][1] = rows[3][2] = 0.0f;
        rows[3][3] = 1.0f;
    } else {  // w = view depth along c; z (unused here) = near
        for (int j = 0; j < 4; j++) rows[3][j] = rows[2][j];
        rows[2][0] = rows[2][1] = rows[2][2] = 0.0f;
        rows[2][3] = 0.1f;
    }
    for (int i = 0; i < 3; i++) {
        vf.a[i] = a[i];
        vf.b[i] = b[i];
        vf.c[i] = c[i];
        vf.e[i] = e[i];
    }
    vf.sx = sx;
    vf.sy = sy;
    lh_mat4 m;
    for (int j = 0; j < 4; j++) {
        m.cols[j].x = rows[0][j];
        m.cols[j].y = rows[1][j];
        m.cols[j].z = rows[2][j];
        m.cols[j].w = rows[3][j];
    }
    return m;
}

int main() {
    std::mt19937_64 rng(5);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    long long tested = 0, skipped = 0, bad = 0, near_tested = 0, near_skipped = 0;
    for (int it = 0; it < 400000; it++) {
        const bool ortho = (it & 1) != 0;
        float Wf, Hf;
        ViewFrame vf;
        const lh_mat4 m = make_view(rng, ortho, Wf, Hf, vf);
        const uint32_t W = (uint32_t)Wf, H = (uint32_t)Hf;
        float c[3], R;
        if (it % 4 < 2) {
            // anywhere, any size
            R = std::pow(10.0f, -3.0f + 4.7f * (U(rng) + 1.0f) * 0.5f);
            for (int i = 0; i < 3; i++) c[i] = U(rng) * 800.0f;
        } else {
            // in front of the view near a pixel, from a hundredth of a pixel to
            // two pixels across
            const float depth = std::pow(10.0f, -0.3f + 3.8f * (U(rng) + 1.0f) * 0.5f);
            const float ox = U(rng), oy = U(rng);
            const float px = ortho ? 2.0f / (Wf * vf.sx) : 2.0f * depth / (Wf * vf.sx);
            R = px * std::pow(10.0f, -2.0f + 2.3f * (U(rng) + 1.0f) * 0.5f);
            for (int i = 0; i < 3; i++) {
                if (ortho)
                    c[i] = vf.e[i] + vf.a[i] * (ox / vf.sx) + vf.b[i] * (oy / vf.sy) + vf.c[i] * depth;
                else
                    c[i] = vf.e[i] + depth * (vf.c[i] + vf.a[i] * (ox / vf.sx) + vf.b[i] * (oy / vf.sy));
            }
        }
        const bool miss = lh::sphere_misses_centres(m, c[0], c[1], c[2], R, W, H);
        tested++;
        near_tested += it % 4 >= 2;
        if (!miss) continue;
        skipped++;
        near_skipped += it % 4 >= 2;
        // sample the box; the raster's transform and snap
        // (64-bit: points far outside the guard band, which the raster clips
        // to pieces inside the same projected box, would not fit 32 bits)
        int64_t minX = INT64_MAX, maxX = INT64_MIN, minY = INT64_MAX, maxY = INT64_MIN;
        bool behind = false;
        for (int k = 0; k < 64; k++) {
            float p[3];
            for (int i = 0; i < 3; i++) {
                const float t = k < 8 ? ((k >> i) & 1 ? 1.0f : -1.0f) : U(rng);
                p[i] = c[i] + t * R;
            }
            auto row = [&](int r) {
                auto el = [&](int col) {
                    const lh_vec4& v = m.cols[col];
                    return r == 0 ? v.x : (r == 1 ? v.y : (r == 2 ? v.z : v.w));
                };
                return ((el(0) * p[0] + el(1) * p[1]) + el(2) * p[2]) + el(3);
            };
            const float x = row(0), y = row(1), w = row(3);
            if (!(w > 0.0f)) {
                behind = true;
                break;
            }
            const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
            const float xf = (x / w) * hw + hw, yf = (y / w) * hh + hh;
            const int64_t X = std::llrint((double)xf * 256.0), Y = std::llrint((double)yf * 256.0);
            minX = X < minX ? X : minX;
            maxX = X > maxX ? X : maxX;
            minY = Y < minY ? Y : minY;
            maxY = Y > maxY ? Y : maxY;
        }
        auto has_centre = [](int64_t lo, int64_t hi, uint32_t n) {
            // centre i at i * 256 + 128, i in [0, n)
            const int64_t first = std::max<int64_t>((lo - 128 + 255) >> 8, 0);
            const int64_t last = std::min<int64_t>((hi - 128) >> 8, (int64_t)n - 1);
            return first <= last;
        };
        if (behind || (has_centre(minX, maxX, W) && has_centre(minY, maxY, H))) {
            if (bad < 10)
                std::printf("it %d: skipped but reaches a centre (behind %d, X %lld..%lld, Y %lld..%lld, R %g)\n", it,
                            (int)behind, (long long)minX, (long long)maxX, (long long)minY, (long long)maxY, R);
            bad++;
        }
    }
    std::printf("tested %lld skipped %lld (near a pixel: %lld of %lld) bad %lld\n", tested, skipped, near_skipped,
                near_tested, bad);
    return bad == 0 && near_skipped > 1000 ? 0 : 1;
}
