// Host driver for the exact stencil sums of cns_exact.cuh: reads lines of eight taps (f[+1..+4],
// f[-1..-4]) as 16-digit hex bit patterns, prints for the first- and the second-derivative
// weights "ok bits" (ok = 0 when the sum takes the FP64 fallback).  Built and run by
// tests/test_exact_sum.py.
#include <cstdio>
#include <cstring>

#include "cns_exact.cuh"

int main() {
    unsigned long long u[8];
    while (scanf("%llx %llx %llx %llx %llx %llx %llx %llx", &u[0], &u[1], &u[2], &u[3], &u[4], &u[5], &u[6],
                 &u[7]) == 8) {
        double t[9];
        for (int m = 0; m < 4; m++) {
            memcpy(&t[4 + m + 1], &u[m], 8);
            memcpy(&t[4 - m - 1], &u[4 + m], 8);
        }
        t[4] = 0.0;
        const double* c = t + 4;
        auto ld = [&](int m) { return c[m]; };
        double x1 = 0.0, x2 = 0.0;
        const bool ok1 = cns::xsum8<672, -168, 32, -3, -1>(ld, &x1);
        const bool ok2 = cns::xsum8<8064, -1008, 128, -9, 1>(ld, &x2);
        unsigned long long b1, b2;
        memcpy(&b1, &x1, 8);
        memcpy(&b2, &x2, 8);
        printf("%d %016llx %d %016llx\n", ok1 ? 1 : 0, ok1 ? b1 : 0ull, ok2 ? 1 : 0, ok2 ? b2 : 0ull);
    }
    return 0;
}
