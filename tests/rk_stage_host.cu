// Host driver for cns_exact.cuh's quarter(), which carries the first RK3 stage between stages as
// U1 / 4: reads lines "x dt r" (16-digit hex bit patterns) and prints the bits of quarter(x) and
// whether fma(dt / 4, r, quarter(x)) has the bits of 0.25 * fma(dt, r, x), the second stage's
// combine as the reference forms it.  Built and run by tests/test_rk_stage.py.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "cns_exact.cuh"

static unsigned long long bits_of(double v) {
    unsigned long long u;
    memcpy(&u, &v, 8);
    return u;
}

int main() {
    unsigned long long ux, ud, ur;
    while (scanf("%llx %llx %llx", &ux, &ud, &ur) == 3) {
        double x, dt, r;
        memcpy(&x, &ux, 8);
        memcpy(&dt, &ud, 8);
        memcpy(&r, &ur, 8);
        const double q = cns::quarter(x);
        const double a = std::fma(0.25 * dt, r, q), b = 0.25 * std::fma(dt, r, x);
        printf("%016llx %d\n", bits_of(q), bits_of(a) == bits_of(b) ? 1 : 0);
    }
    return 0;
}
