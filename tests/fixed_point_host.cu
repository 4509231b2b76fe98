// Host driver for the fixed-point stencil copies of cns_exact.cuh: reads lines "E t1..t8" (E a
// decimal exponent, the taps f[+1..+4], f[-1..-4] as 16-digit hex bit patterns) and prints the
// eight fixed-point words, the flag of a value that did not fit, and for the first- and the
// second-derivative weights "ok bits" of the rounded sums; then "ok bits" of the merged
// second-difference sums over two and three stencils: the words as given, mirrored (tap m read
// at -m) and rotated (tap m read at the next m).  Built and run by tests/test_fixed_point.py.
#include <cstdio>
#include <cstring>

#include "cns_exact.cuh"

int main() {
    int E;
    unsigned long long u[8];
    while (scanf("%d %llx %llx %llx %llx %llx %llx %llx %llx", &E, &u[0], &u[1], &u[2], &u[3], &u[4], &u[5], &u[6],
                 &u[7]) == 9) {
        long long w[9];
        bool bad = false;
        for (int m = 0; m < 4; m++) {
            double a, b;
            memcpy(&a, &u[m], 8);
            memcpy(&b, &u[4 + m], 8);
            w[4 + m + 1] = cns::fx_word(a, E, &bad);
            w[4 - m - 1] = cns::fx_word(b, E, &bad);
        }
        w[4] = 0;
        const long long* c = w + 4;
        auto ld = [&](int m) { return c[m]; };
        double x1 = 0.0, x2 = 0.0;
        const bool ok1 = cns::fx_sum8<672, -168, 32, -3, -1>(ld, E, &x1);
        const bool ok2 = cns::fx_sum8<8064, -1008, 128, -9, 1>(ld, E, &x2);
        unsigned long long b1, b2;
        memcpy(&b1, &x1, 8);
        memcpy(&b2, &x2, 8);
        auto mir = [&](int m) { return c[-m]; };
        auto rot = [&](int m) { return c[m > 0 ? (m % 4) + 1 : -((-m % 4) + 1)]; };
        const double one[5] = {0.0, 0.0, 0.0, 0.0, 1.0};
        bool f2 = false, f3 = false;
        const double x22 = cns::fx_d2acc2(0.0, ld, mir, E, one, &f2);
        const double x23 = cns::fx_d2acc3(0.0, ld, mir, rot, E, one, &f3);
        unsigned long long b22, b23;
        memcpy(&b22, &x22, 8);
        memcpy(&b23, &x23, 8);
        for (int m = 1; m <= 4; m++) printf("%016llx ", (unsigned long long)c[m]);
        for (int m = 1; m <= 4; m++) printf("%016llx ", (unsigned long long)c[-m]);
        printf("%d %d %016llx %d %016llx %d %016llx %d %016llx\n", bad ? 1 : 0, ok1 ? 1 : 0, ok1 ? b1 : 0ull,
               ok2 ? 1 : 0, ok2 ? b2 : 0ull, f2 ? 0 : 1, f2 ? 0ull : b22, f3 ? 0 : 1, f3 ? 0ull : b23);
    }
    return 0;
}
