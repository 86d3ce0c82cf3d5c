// Host check of lighthugger_gb300/csrc/edge_run.cuh: for random triangles
// (snapped 1/256-pixel coordinates from a few pixels across up to the
// guard band's extent), random chunk rectangles of up to 32 x 256 pixels
// and every top-left bias, the intersection of the three edges' runs must
// hold exactly the pixels whose three integer edge functions pass their
// tests, row by row.
#include <cstdio>
#include <random>

#include "edge_run.cuh"

static int64_t edge_at(int32_t ax, int32_t ay, int32_t bx, int32_t by, int32_t px, int32_t py) {
    return (int64_t)(by - ay) * ((int64_t)px * 256 + 128 - ax) - (int64_t)(bx - ax) * ((int64_t)py * 256 + 128 - ay);
}

int main() {
    std::mt19937_64 rng(11);
    long long rows_checked = 0, bad = 0, covered = 0;
    const int32_t scales[] = {4, 40, 400, 4000, 60000, 1 << 19};  // pixels
    for (int it = 0; it < 300000; it++) {
        const int32_t sc = scales[it % 6];
        auto coord = [&](int32_t c) { return (int32_t)(c * 256 + (int64_t)(rng() % (2ull * sc * 256)) - (int64_t)sc * 256); };
        const int32_t cx = (int32_t)(rng() % 2000), cy = (int32_t)(rng() % 2000);
        int32_t X[3], Y[3];
        for (int k = 0; k < 3; k++) {
            X[k] = coord(cx);
            Y[k] = coord(cy);
        }
        if (it % 7 == 0) X[1] = X[0];  // axis-aligned edges
        if (it % 11 == 0) Y[2] = Y[1];
        const uint32_t bias = (uint32_t)(rng() & 7u);
        const int32_t n = 1 + (int32_t)(rng() % 256), rows = 1 + (int32_t)(rng() % 32);
        // a chunk near the triangle: around a vertex or the centroid
        const int k0 = (int)(rng() % 4);
        const int32_t ax = k0 < 3 ? X[k0] / 256 : (X[0] + X[1] + X[2]) / 768;
        const int32_t ay = k0 < 3 ? Y[k0] / 256 : (Y[0] + Y[1] + Y[2]) / 768;
        const int32_t x0 = ax - (int32_t)(rng() % (uint32_t)n), y0 = ay - (int32_t)(rng() % (uint32_t)rows);
        const int32_t E[3][4] = {{X[1], Y[1], X[2], Y[2]}, {X[2], Y[2], X[0], Y[0]}, {X[0], Y[0], X[1], Y[1]}};
        for (int32_t r = 0; r < rows; r++) {
            const int32_t y = y0 + r;
            int32_t lo = 0, hi = n - 1;
            for (int e = 0; e < 3; e++) {
                const int32_t dy = E[e][3] - E[e][1];
                lh::clip_run(edge_at(E[e][0], E[e][1], E[e][2], E[e][3], x0, y), (int64_t)dy * 256, (bias >> e) & 1u, n,
                             lh::run_inv_step(dy), lo, hi);
            }
            rows_checked++;
            for (int32_t k = 0; k < n; k++) {
                bool in = true;
                for (int e = 0; e < 3; e++)
                    in = in && edge_at(E[e][0], E[e][1], E[e][2], E[e][3], x0 + k, y) >= (int64_t)((bias >> e) & 1u);
                const bool run = k >= lo && k <= hi;
                covered += in;
                if (in != run) {
                    if (bad < 10)
                        std::printf("it %d row %d k %d: pixel %d run [%d, %d] n %d\n", it, r, k, (int)in, lo, hi, n);
                    bad++;
                    break;
                }
            }
        }
    }
    std::printf("rows %lld covered %lld bad %lld\n", rows_checked, covered, bad);
    return bad == 0 ? 0 : 1;
}
