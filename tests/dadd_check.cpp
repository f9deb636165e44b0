// Host build of the walk's integer double addition (sw_dadd.h) against the host's IEEE double
// addition: positions + Gaussian steps, cancellation and rounding ties at nearby exponents,
// random bit patterns over the whole range (specials included). Prints the mismatch count.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "sw_dadd.h"

int main(int argc, char **argv) {
    const long iters = argc > 1 ? atol(argv[1]) : 1000000;
    std::mt19937_64 r(7);
    std::uniform_real_distribution<double> U(0, 1);
    long bad = 0, n = 0;
    auto chk = [&](double a, double b) {
        const double x = sw::dadd_int(a, b), y = a + b;
        n++;
        if (sw::dbits(x) != sw::dbits(y)) {
            if (bad < 5) printf("a=%a b=%a got %a want %a\n", a, b, x, y);
            bad++;
        }
    };
    for (long i = 0; i < iters; i++) {
        const double x = U(r) * 5e-4, g = (U(r) - 0.5) * 8e-7;
        chk(x, g);
        chk(g, x);
        chk(-x, g);
        const uint64_t ua = r(), ub = r(), ea = 900 + r() % 200, eb = ea - r() % 70 + 3;
        const double a = sw::dfrom((ua & 0x800fffffffffffffull) | (ea << 52));
        const double b = sw::dfrom((ub & 0x800fffffffffffffull) | (eb << 52));
        chk(a, b);
        chk(a, -a);
        chk(a, -b);
        chk(a, sw::dfrom((ub & 0x8000000000000000ull) | ((ea - 53 + r() % 3) << 52)));
        chk(sw::dfrom(r()), sw::dfrom(r()));
        if (sw::dtwice_abs(sw::dbits(g)) != sw::dbits(2 * std::fabs(g)) ||
            sw::dflip(sw::dbits(a)) != sw::dbits(-a))
            bad++;
    }
    chk(0.0, 1.0);
    chk(-0.0, 0.0);
    chk(1e-310, 1.0);
    chk(INFINITY, 1.0);
    chk(1.0, -1.0);
    printf("%ld %ld\n", n, bad);
    return bad != 0;
}
