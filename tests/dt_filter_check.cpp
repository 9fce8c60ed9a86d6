// Check of the dt pass's single-precision filter (point.cuh): for random
// nodes — depths from films to the deep ocean, velocities of either sign
// and of any size up to 50 m/s, metrics of either sign and of any element
// size, and rates where u·m0 and v·m1 nearly cancel — the float rate lies
// within 2^-20·B of the double rate (B its error scale), and the filter
// never drops the node holding an element's largest rate. Built for the
// host with the IEEE arithmetic; prints one line, exits 1 on failure.
#define DGSWE_FAST 0
#define DGSWE_NS exact
#include <cmath>
#include <cstdio>
#include <random>

#include "point.cuh"

using namespace dgswe;
using namespace dgswe::exact;

static std::mt19937_64 rng(20261204);
static double uni(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }
static double logu(double a, double b) { return std::exp(uni(std::log(a), std::log(b))); }

int main() {
    const double g = 9.81;
    const float g32 = f32_trunc(g);
    long checked = 0, failed = 0, dropped = 0;
    double worst = 0.0;
    for (int element = 0; element < 200000; ++element) {
        // one element's 32 rate slots with a common scale, as an element's are
        const double size = logu(1.0, 5e4);
        double r64[32];
        float r32[32], b32[32];
        for (int s = 0; s < 32; ++s) {
            double m[6];
            for (int c = 0; c < 4; ++c) m[c] = uni(-1.0, 1.0) / size;
            m[4] = std::sqrt(m[0] * m[0] + m[1] * m[1]);
            m[5] = std::sqrt(m[2] * m[2] + m[3] * m[3]);
            const double h = logu(1e-6, 500.0);
            double u = uni(-1.0, 1.0) * logu(1e-9, 50.0), v = uni(-1.0, 1.0) * logu(1e-9, 50.0);
            if (s % 4 == 1 && std::fabs(m[1]) > 0.0) v = -u * m[0] / m[1] * (1.0 + uni(-1e-7, 1e-7));
            r64[s] = node_rate(h, u, v, m, g);
            float m32[6];  // the library's float table: each value truncated
            for (int c = 0; c < 6; ++c) m32[c] = f32_trunc(m[c]);
            node_rate_f32(h, u, v, m32, g32, r32[s], b32[s]);
            const double err = std::fabs(r64[s] - (double)r32[s]);
            const double bound = std::ldexp((double)b32[s], -20) * (1.0 + 1e-6) + 1e-37;
            ++checked;
            if (!(err <= bound)) {
                if (++failed <= 5)
                    std::printf("bound broken: h %.17g u %.17g v %.17g r64 %.17g r32 %.9g B %.9g\n",
                                h, u, v, r64[s], (double)r32[s], (double)b32[s]);
            }
            worst = std::fmax(worst, bound > 0.0 ? err / bound : 0.0);
        }
        // the kernel's filter: δ = 2^-16, floor 1e-30
        const float delta = 1.0f / 65536.0f;
        float thr = 0.0f;
        int arg = 0;
        for (int s = 0; s < 32; ++s) {
            thr = std::fmax(thr, std::fmax(r32[s] - (delta * b32[s] + 1e-30f), 0.0f));
            if (r64[s] > r64[arg]) arg = s;
        }
        if (!(r32[arg] + (delta * b32[arg] + 1e-30f) >= thr)) ++dropped;
    }
    std::printf("%s %ld rates, %ld beyond the bound, %ld maxima dropped, worst %.3f of the bound\n",
                failed || dropped ? "FAIL" : "ok", checked, failed, dropped, worst);
    return failed || dropped ? 1 : 0;
}
