// CPU check of the hand-written adjoint in lighthugger_gb300/csrc/shade.cuh:
// random pixels, analytic gradient (double) against central differences of
// the same forward (double, h = 1e-5 relative).  Parameters whose difference
// quotient is not smooth at h (a clamp, a texel centre, a flipped compare or
// face sign within h) are skipped: the quotients at h and h/2 must agree.
// Prints the number of checked parameters and the worst relative error;
// exits 1 above the tolerance.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "shade.cuh"

using namespace lh::shade;

struct HostSampler {
    int tw = 8, th = 8;
    std::vector<double> tex[2];  // base (rgb linear), mr
    int S = 16;
    std::vector<double> shadow;  // 4 layers
    Bilinear<double> sample(uint32_t index, v2<double> uv) const {
        const std::vector<double>& t = tex[index];
        Bilinear<double> s;
        double u = uv.x * tw - 0.5, v = uv.y * th - 0.5;
        double fu = std::floor(u), fv = std::floor(v);
        s.a = u - fu;
        s.b = v - fv;
        int32_t i0 = (int32_t)fu, j0 = (int32_t)fv;
        auto wrap = [](int32_t i, int32_t n) { return ((i % n) + n) % n; };
        s.i0 = wrap(i0, tw); s.i1 = wrap(i0 + 1, tw); s.j0 = wrap(j0, th); s.j1 = wrap(j0 + 1, th);
        for (int c = 0; c < 4; c++) {
            s.t00[c] = t[(s.j0 * tw + s.i0) * 4 + c];
            s.t10[c] = t[(s.j0 * tw + s.i1) * 4 + c];
            s.t01[c] = t[(s.j1 * tw + s.i0) * 4 + c];
            s.t11[c] = t[(s.j1 * tw + s.i1) * 4 + c];
        }
        s.size_u = tw;
        s.size_v = th;
        s.index = index;
        return s;
    }
    double shadow_cmp(uint32_t layer, int32_t i, int32_t j, double ref) const {
        i = i < 0 ? 0 : (i > S - 1 ? S - 1 : i);
        j = j < 0 ? 0 : (j > S - 1 ? S - 1 : j);
        return ref < shadow[(layer * S + j) * S + i] ? 1.0 : 0.0;
    }
};

int main(int argc, char** argv) {
    int pixels = argc > 1 ? atoi(argv[1]) : 300;
    std::mt19937_64 rng(1234);
    std::uniform_real_distribution<double> U(-1, 1), U01(0, 1);
    HostSampler smp;
    for (int t = 0; t < 2; t++) {
        smp.tex[t].resize(smp.tw * smp.th * 4);
        for (auto& x : smp.tex[t]) x = 0.1 + 0.8 * U01(rng);
    }
    smp.shadow.resize(4 * smp.S * smp.S);
    for (auto& x : smp.shadow) x = U01(rng) < 0.5 ? 0.3 : 0.9;
    long checked = 0, skipped = 0, bad = 0, nontrivial = 0;
    double worst = 0;
    for (int px = 0; px < pixels; px++) {
        PixelFixed fx = {};
        // camera looking down -z at a triangle around z = -5; perspective-like PV
        double f = 1.7;
        float pv[4][4] = {{(float)(f / 1.5), 0, 0, 0}, {0, (float)-f, 0, 0}, {0, 0, 0, -1}, {0, 0, 0.01f, 0}};
        for (int c = 0; c < 4; c++) for (int r = 0; r < 4; r++) fx.pv[c][r] = pv[c][r];
        for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) fx.nt[c][r] = (c == r ? 1.0f : 0.0f) + 0.2f * (float)U(rng);
        // orthographic uv-space shadow matrix: uv = 0.5 + world.xy * s
        float s = 0.05f;
        float uvs[4][4] = {{s, 0, 0, 0}, {0, s, 0, 0}, {0, 0, 0.01f, 0}, {0.5f, 0.5f, 0.5f, 1}};
        for (int c = 0; c < 4; c++) for (int r = 0; r < 4; r++) fx.uvs[c][r] = uvs[c][r];
        fx.cam[0] = fx.cam[1] = fx.cam[2] = 0;
        fx.ndc[0] = (float)(0.3 * U(rng));
        fx.ndc[1] = (float)(0.3 * U(rng));
        fx.win[0] = 640; fx.win[1] = 480;
        fx.ts[0] = fx.ts[1] = 1; fx.toff[0] = fx.toff[1] = 0;
        fx.bias = 0;
        fx.shadow_size = (float)smp.S;
        fx.cascade = (uint32_t)(rng() % 4);
        fx.thin = (uint32_t)(rng() % 2);
        fx.base_tex = 0; fx.mr_tex = 1;
        PixelParams<double> p;
        // a triangle around the pixel's ray at depth ~5
        double z = -5 + U(rng);
        double cx = fx.ndc[0] * 1.5 / f * -z, cy = -fx.ndc[1] / f * -z;
        for (int k = 0; k < 3; k++) {
            double ang = 2.1 * k + 0.3 * U(rng);
            p.W[k] = {cx + 1.5 * std::cos(ang), cy + 1.5 * std::sin(ang), z + 0.5 * U(rng)};
            p.N[k] = {0.3 * U(rng), 0.3 * U(rng), 1.0 + 0.2 * U(rng)};
            p.UV[k] = {U01(rng), U01(rng)};
        }
        p.bcf = {0.5 + 0.5 * U01(rng), 0.5 + 0.5 * U01(rng), 0.5 + 0.5 * U01(rng)};
        p.sun = normalize(v3<double>{0.3 * U(rng), 0.5 * U(rng), 1.0});
        p.light = {0.5 + U01(rng), 0.5 + U01(rng), 0.5 + U01(rng)};
        v3<double> gout{U(rng), U(rng), U(rng)};
        v3<double> val;
        PixelGrad<double> g;
        decide(fx, p, smp);
        shade(fx, p, smp, &val, gout, &g);
        auto loss = [&](const PixelParams<double>& q, const HostSampler& sm) {
            v3<double> o;
            PixelFixed fq = fx;
            decide(fq, q, sm);  // the decisions at the perturbed point (jumps are skipped)
            shade<double>(fq, q, sm, &o, gout, nullptr);
            return (o.x * gout.x + o.y * gout.y) + o.z * gout.z;
        };
        auto check = [&](double analytic, auto&& perturb) {
            double h = 1e-5;
            double fd1 = (perturb(h) - perturb(-h)) / (2 * h);
            double fd2 = (perturb(h / 2) - perturb(-h / 2)) / h;
            double scale = std::fabs(fd1) + std::fabs(fd2) + 1e-6;
            if (std::fabs(fd1 - fd2) > 1e-4 * scale + 1e-9) { skipped++; return; }
            double err = std::fabs(analytic - fd1) / (std::fabs(fd1) + 1e-4);
            checked++;
            if (std::fabs(fd1) > 1e-3) nontrivial++;
            if (err > worst) worst = err;
            if (err > 1e-3) {
                bad++;
                if (bad < 10) std::printf("mismatch: analytic %.9g fd %.9g\n", analytic, fd1);
            }
        };
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) {
                double* gw = c == 0 ? &g.W[k].x : c == 1 ? &g.W[k].y : &g.W[k].z;
                check(*gw, [&](double h) {
                    PixelParams<double> q = p;
                    double* x = c == 0 ? &q.W[k].x : c == 1 ? &q.W[k].y : &q.W[k].z;
                    *x += h;
                    return loss(q, smp);
                });
                double* gn = c == 0 ? &g.N[k].x : c == 1 ? &g.N[k].y : &g.N[k].z;
                check(*gn, [&](double h) {
                    PixelParams<double> q = p;
                    double* x = c == 0 ? &q.N[k].x : c == 1 ? &q.N[k].y : &q.N[k].z;
                    *x += h;
                    return loss(q, smp);
                });
            }
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 2; c++) {
                check(c == 0 ? g.UV[k].x : g.UV[k].y, [&](double h) {
                    PixelParams<double> q = p;
                    (c == 0 ? q.UV[k].x : q.UV[k].y) += h;
                    return loss(q, smp);
                });
            }
        for (int c = 0; c < 3; c++) {
            check(c == 0 ? g.bcf.x : c == 1 ? g.bcf.y : g.bcf.z, [&](double h) {
                PixelParams<double> q = p;
                (c == 0 ? q.bcf.x : c == 1 ? q.bcf.y : q.bcf.z) += h;
                return loss(q, smp);
            });
            check(c == 0 ? g.sun.x : c == 1 ? g.sun.y : g.sun.z, [&](double h) {
                PixelParams<double> q = p;
                (c == 0 ? q.sun.x : c == 1 ? q.sun.y : q.sun.z) += h;
                return loss(q, smp);
            });
            check(c == 0 ? g.light.x : c == 1 ? g.light.y : g.light.z, [&](double h) {
                PixelParams<double> q = p;
                (c == 0 ? q.light.x : c == 1 ? q.light.y : q.light.z) += h;
                return loss(q, smp);
            });
        }
        // texels used by the bilinear samples
        Bilinear<double> sb;
        {
            // sample position from the forward: find it by re-running with a probing sampler
            struct Probe : HostSampler {
                mutable v2<double> last[2];
                Bilinear<double> sample(uint32_t index, v2<double> uv) const {
                    last[index] = uv;
                    return HostSampler::sample(index, uv);
                }
            } probe;
            static_cast<HostSampler&>(probe) = smp;
            v3<double> o;
            PixelFixed fq = fx;
            decide(fq, p, probe);
            shade<double>(fq, p, probe, &o, gout, nullptr);
            sb = smp.sample(0, probe.last[0]);
            Bilinear<double> sm = smp.sample(1, probe.last[1]);
            int64_t ti[4] = {(int64_t)sb.j0 * smp.tw + sb.i0, (int64_t)sb.j0 * smp.tw + sb.i1,
                             (int64_t)sb.j1 * smp.tw + sb.i0, (int64_t)sb.j1 * smp.tw + sb.i1};
            int64_t tm[4] = {(int64_t)sm.j0 * smp.tw + sm.i0, (int64_t)sm.j0 * smp.tw + sm.i1,
                             (int64_t)sm.j1 * smp.tw + sm.i0, (int64_t)sm.j1 * smp.tw + sm.i1};
            bool dup_b = false, dup_m = false;
            for (int a = 0; a < 4; a++)
                for (int b = a + 1; b < 4; b++) { dup_b |= ti[a] == ti[b]; dup_m |= tm[a] == tm[b]; }
            for (int q = 0; q < 4 && !dup_b; q++)
                for (int c = 0; c < 3; c++)
                    check(g.base_texel[q][c], [&](double h) {
                        HostSampler s2 = smp;
                        s2.tex[0][ti[q] * 4 + c] += h;
                        return loss(p, s2);
                    });
            for (int q = 0; q < 4 && !dup_m; q++)
                for (int c = 0; c < 2; c++)
                    check(g.mr_texel[q][c], [&](double h) {
                        HostSampler s2 = smp;
                        s2.tex[1][tm[q] * 4 + 1 + c] += h;
                        return loss(p, s2);
                    });
        }
    }
    // float32 against float64 at world-scale coordinates (everything moved
    // ~400 m from the origin): the precision the GPU kernel works at.
    struct FloatSampler {
        const HostSampler* h;
        Bilinear<float> sample(uint32_t index, v2<float> uv) const {
            Bilinear<double> d = h->sample(index, v2<double>{uv.x, uv.y});
            Bilinear<float> f;
            for (int c = 0; c < 4; c++) {
                f.t00[c] = (float)d.t00[c]; f.t10[c] = (float)d.t10[c];
                f.t01[c] = (float)d.t01[c]; f.t11[c] = (float)d.t11[c];
            }
            f.a = (float)(uv.x * h->tw - 0.5f - std::floor(uv.x * h->tw - 0.5f));
            f.b = (float)(uv.y * h->th - 0.5f - std::floor(uv.y * h->th - 0.5f));
            f.size_u = (float)h->tw; f.size_v = (float)h->th;
            f.i0 = d.i0; f.i1 = d.i1; f.j0 = d.j0; f.j1 = d.j1; f.index = d.index;
            return f;
        }
        float shadow_cmp(uint32_t layer, int32_t i, int32_t j, float ref) const {
            return (float)h->shadow_cmp(layer, i, j, ref);
        }
    };
    FloatSampler fsmp{&smp};
    double worst_f32 = 0;
    long f32_checked = 0;
    for (int px = 0; px < pixels; px++) {
        PixelFixed fx = {};
        double f = 1.7;
        const double off[3] = {300.0, 40.0, -250.0};
        // P V with the eye at `off`: clip = P (world - off)
        float P[4][4] = {{(float)(f / 1.5), 0, 0, 0}, {0, (float)-f, 0, 0}, {0, 0, 0, -1}, {0, 0, 0.01f, 0}};
        for (int c = 0; c < 4; c++) for (int r = 0; r < 4; r++) fx.pv[c][r] = P[c][r];
        for (int r = 0; r < 4; r++)
            fx.pv[3][r] = (float)((double)P[3][r] - (P[0][r] * off[0] + P[1][r] * off[1] + P[2][r] * off[2]));
        for (int c = 0; c < 3; c++) for (int r = 0; r < 3; r++) fx.nt[c][r] = (c == r ? 1.0f : 0.0f);
        float sc = 0.05f;
        float uvs[4][4] = {{sc, 0, 0, 0}, {0, sc, 0, 0}, {0, 0, 0.01f, 0},
                           {(float)(0.5 - sc * off[0]), (float)(0.5 - sc * off[1]), 0.5f, 1}};
        for (int c = 0; c < 4; c++) for (int r = 0; r < 4; r++) fx.uvs[c][r] = uvs[c][r];
        fx.cam[0] = (float)off[0]; fx.cam[1] = (float)off[1]; fx.cam[2] = (float)off[2];
        fx.ndc[0] = (float)(0.3 * U(rng)); fx.ndc[1] = (float)(0.3 * U(rng));
        fx.win[0] = 640; fx.win[1] = 480;
        fx.ts[0] = fx.ts[1] = 1;
        fx.shadow_size = (float)smp.S;
        fx.cascade = 1;
        fx.base_tex = 0; fx.mr_tex = 1;
        PixelParams<double> p;
        double z = -8 + U(rng);
        double cx = fx.ndc[0] * 1.5 / f * -z, cy = -fx.ndc[1] / f * -z;
        for (int k = 0; k < 3; k++) {
            double ang = 2.1 * k + 0.3 * U(rng);
            p.W[k] = {off[0] + cx + 0.3 * std::cos(ang), off[1] + cy + 0.3 * std::sin(ang), off[2] + z + 0.1 * U(rng)};
            p.N[k] = {0.3 * U(rng), 0.3 * U(rng), 1.0};
            p.UV[k] = {U01(rng), U01(rng)};
        }
        p.bcf = {0.8, 0.7, 0.6};
        p.sun = normalize(v3<double>{0.3, 0.4, 1.0});
        p.light = {1, 1, 1};
        // round the inputs to float first, so both precisions see the same values
        PixelParams<float> pf;
        for (int k = 0; k < 3; k++) {
            pf.W[k] = {(float)p.W[k].x, (float)p.W[k].y, (float)p.W[k].z};
            p.W[k] = {pf.W[k].x, pf.W[k].y, pf.W[k].z};
            pf.N[k] = {(float)p.N[k].x, (float)p.N[k].y, (float)p.N[k].z};
            p.N[k] = {pf.N[k].x, pf.N[k].y, pf.N[k].z};
            pf.UV[k] = {(float)p.UV[k].x, (float)p.UV[k].y};
            p.UV[k] = {pf.UV[k].x, pf.UV[k].y};
        }
        pf.bcf = {(float)p.bcf.x, (float)p.bcf.y, (float)p.bcf.z};
        pf.sun = {(float)p.sun.x, (float)p.sun.y, (float)p.sun.z};
        p.sun = {pf.sun.x, pf.sun.y, pf.sun.z};
        pf.light = {1, 1, 1};
        v3<double> gout{U(rng), U(rng), U(rng)};
        v3<double> vd;
        v3<float> vf;
        PixelGrad<double> gd;
        PixelGrad<float> gf;
        decide(fx, p, smp);
        shade(fx, p, smp, &vd, gout, &gd);
        // the float pass in camera-relative coordinates, as the GPU kernel runs it
        PixelFixed fr = fx;
        double cam[3] = {fx.cam[0], fx.cam[1], fx.cam[2]};
        for (int r = 0; r < 4; r++) {
            fr.pv[3][r] = (float)((double)fx.pv[3][r] + ((double)fx.pv[0][r] * cam[0] + (double)fx.pv[1][r] * cam[1] +
                                                         (double)fx.pv[2][r] * cam[2]));
            fr.uvs[3][r] = (float)((double)fx.uvs[3][r] + ((double)fx.uvs[0][r] * cam[0] +
                                                           (double)fx.uvs[1][r] * cam[1] + (double)fx.uvs[2][r] * cam[2]));
        }
        fr.cam[0] = fr.cam[1] = fr.cam[2] = 0.0f;
        for (int k = 0; k < 3; k++)
            pf.W[k] = {pf.W[k].x - fx.cam[0], pf.W[k].y - fx.cam[1], pf.W[k].z - fx.cam[2]};
        shade<float>(fr, pf, fsmp, &vf, v3<float>{(float)gout.x, (float)gout.y, (float)gout.z}, &gf);
        double scale = 0;
        for (int k = 0; k < 3; k++)
            scale = std::max(scale, std::max(std::fabs(gd.W[k].x), std::max(std::fabs(gd.W[k].y), std::fabs(gd.W[k].z))));
        for (int k = 0; k < 3; k++) {
            double e = std::max(std::fabs(gf.W[k].x - gd.W[k].x),
                                std::max(std::fabs(gf.W[k].y - gd.W[k].y), std::fabs(gf.W[k].z - gd.W[k].z)));
            worst_f32 = std::max(worst_f32, e / (scale + 1e-12));
            f32_checked++;
        }
    }
    std::printf("f32 position gradients at world scale: %ld checked, worst error %.3g of the pixel's largest\n",
                f32_checked, worst_f32);
    if (worst_f32 > 3e-4) bad++;
    std::printf("checked %ld nontrivial %ld skipped %ld bad %ld worst_rel_err %.3g\n", checked, nontrivial, skipped, bad,
                worst);
    return (bad == 0 && checked > 1000 && nontrivial > checked / 4) ? 0 : 1;
}
