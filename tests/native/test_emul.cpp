// Host unit test of the integer-pipe FP64 multiply (lgpu_f64emu.cuh):
// emul(x, k) must equal the IEEE product x*k except on exact rounding ties
// (then within one ulp), for random and edge-case operands.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "lgpu_f64emu.cuh"

int main() {
    std::mt19937_64 gen(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::uniform_int_distribution<int> ex(-60, 0);
    long exact = 0, oneulp = 0, bad = 0, total = 0;
    auto check = [&](double x, double k) {
        const double ref = x * k;
        const double got = lgpu::emul(x, lgpu::make_kconst(k));
        total++;
        if (got == ref || (ref == 0.0 && got == 0.0)) {
            exact++;
            return;
        }
        if (std::fabs(ref) <= 2.2250738585072014e-308) {  // results at or below 2^-1022 may flush to zero
            if (got == 0.0) { exact++; return; }
        }
        const double ulp = std::fabs(std::nextafter(ref, 2 * ref) - ref);
        if (std::fabs(got - ref) <= ulp) { oneulp++; return; }
        if (bad < 10) std::printf("bad: x=%a k=%a ref=%a got=%a\n", x, k, ref, got);
        bad++;
    };
    for (int i = 0; i < 2000000; i++) check(std::ldexp(u(gen), ex(gen)), std::ldexp(u(gen), ex(gen) / 4));
    const double edge[] = {0.0, -0.0, 1.0, -1.0, 0.5, 0.7071067811865476, -0.7071067811865476, 1e-300, 3e-310,
                           0.9999999999999999, 2.2250738585072014e-308};
    for (double x : edge)
        for (double k : edge) check(x, k);
    std::printf("total %ld exact %ld one-ulp %ld bad %ld\n", total, exact, oneulp, bad);
    return bad == 0 ? 0 : 1;
}
