// Checks every helper of dgcom_gb300/csrc/fp64_bits.hpp against the IEEE
// comparison or select it replaces, on special values (±0, subnormals,
// extremes, infinities), random bit patterns and adjacent-ulp pairs.
// NaN arguments are excluded: the helpers promise IEEE results for every
// other double. Prints the number of checks; exits 1 on the first mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "fp64_bits.hpp"

using namespace dgswe;

static uint64_t u(double x) {
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
}
static double d(uint64_t b) {
    double x;
    std::memcpy(&x, &b, 8);
    return x;
}

static long checks = 0;
static int fail(const char* what, double a, double b) {
    std::printf("MISMATCH %s a=%a (0x%016llx) b=%a (0x%016llx)\n", what, a, (unsigned long long)u(a),
                b, (unsigned long long)u(b));
    return 1;
}

#define CHECK(cond, what)                    \
    do {                                     \
        ++checks;                            \
        if (!(cond)) return fail(what, a, b); \
    } while (0)

static int pair(double a, double b) {
    CHECK(fp::gt(a, b) == (a > b), "gt");
    CHECK(fp::ge(a, b) == (a >= b), "ge");
    CHECK(fp::lt(a, b) == (a < b), "lt");
    CHECK(fp::le(a, b) == (a <= b), "le");
    CHECK(u(fp::lmax(a, b)) == u(a > b ? a : b), "lmax");
    CHECK(u(fp::lmin(a, b)) == u(a < b ? a : b), "lmin");
    CHECK(fp::gt0(a) == (a > 0.0), "gt0");
    CHECK(fp::le0(a) == (a <= 0.0), "le0");
    CHECK(fp::lt0(a) == (a < 0.0), "lt0");
    CHECK(fp::ge0(a) == (a >= 0.0), "ge0");
    CHECK(fp::nz(a) == (a != 0.0), "nz");
    CHECK(fp::finite(a) == std::isfinite(a), "finite");
    CHECK(u(fp::max0(a)) == u(a > 0.0 ? a : 0.0), "max0");
    if (!std::signbit(a) && !std::signbit(b)) {
        CHECK(fp::gt_nn(a, b) == (a > b), "gt_nn");
        CHECK(u(fp::max_nn(a, b)) == u(a > b ? a : b), "max_nn");
        CHECK(u(fp::min_nn(a, b)) == u(a < b ? a : b), "min_nn");
    }
    return 0;
}

int main() {
    const double inf = std::numeric_limits<double>::infinity();
    std::vector<double> special = {0.0,
                                   -0.0,
                                   d(1),
                                   -d(1),
                                   d(0x000FFFFFFFFFFFFFull),
                                   -d(0x000FFFFFFFFFFFFFull),
                                   std::numeric_limits<double>::min(),
                                   -std::numeric_limits<double>::min(),
                                   1e-300,
                                   -1e-300,
                                   1e-14,
                                   1e-10,
                                   1e-6,
                                   -1e-6,
                                   0.99,
                                   1.0,
                                   -1.0,
                                   1.0000000000000002,
                                   0.9999999999999999,
                                   9.81,
                                   20.0,
                                   -20.0,
                                   std::numeric_limits<double>::max(),
                                   -std::numeric_limits<double>::max(),
                                   inf,
                                   -inf};
    for (double a : special)
        for (double b : special)
            if (pair(a, b)) return 1;
    // NaN is never finite, the one NaN case the helpers define
    if (fp::finite(std::nan(""))) return fail("finite(NaN)", 0, 0);
    std::mt19937_64 rng(20261203);
    auto random_double = [&]() {
        for (;;) {
            double x = d(rng());
            if (!std::isnan(x)) return x;
        }
    };
    for (int n = 0; n < 2000000; ++n) {
        const double a = random_double();
        double b;
        switch (n % 4) {
            case 0: b = random_double(); break;
            case 1: b = std::nextafter(a, inf); break;
            case 2: b = std::nextafter(a, -inf); break;
            default: b = -a; break;
        }
        if (std::isnan(b)) continue;
        if (pair(a, b) || pair(b, a)) return 1;
        const double s = special[n % special.size()];
        if (pair(a, s) || pair(s, a)) return 1;
    }
    std::printf("ok %ld checks\n", checks);
    return 0;
}
