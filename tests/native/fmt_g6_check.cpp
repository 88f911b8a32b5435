// Checks gsnp_gb300/csrc/fmt_g6.h against the C library's printf("%#.6g").
// Prints the number of values compared and exits 1 on the first difference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>

#include "fmt_g6.h"

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next() {
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static long checked = 0;
static bool check(double v, bool must_support) {
    char a[64], b[64];
    const int n = gsnp::fmt_g6(v, a);
    if (n == 0) {
        if (must_support) {
            printf("unsupported %.17g\n", v);
            return false;
        }
        return true;
    }
    a[n] = 0;
    snprintf(b, sizeof(b), "%#.6g", v);
    ++checked;
    if (strcmp(a, b) != 0) {
        printf("mismatch %.17g: got %s want %s\n", v, a, b);
        return false;
    }
    return true;
}

int main() {
    // every copy ratio repeat/depth the cns text can hold for depth <= 1500
    for (int d = 1; d <= 1500; ++d)
        for (int r = 0; r <= 5 * d; ++r)
            if (!check((double)r / d, true)) return 1;
    // random doubles across the supported decades and beyond
    for (int i = 0; i < 4000000; ++i) {
        const double x = std::ldexp((double)(next() >> 11) / 9007199254740992.0 + 0.5, (int)(next() % 140) - 110);
        if (!check(x, x > 1e-26 && x < 9e5)) return 1;
    }
    // values at and next to 6-digit rounding boundaries
    for (int i = 0; i < 2000000; ++i) {
        const int X = (int)(next() % 30) - 24;
        const double base = (double)(100000 + next() % 900000) + 0.5;
        const double v = base * std::pow(10.0, X - 5);
        for (double w : {v, std::nextafter(v, 0.0), std::nextafter(v, 1e300)})
            if (!check(w, w > 1e-26 && w < 9e5)) return 1;
    }
    // dyadic values (exact ties are possible) and specials
    for (int j = 1; j < 60; ++j)
        for (int k = 1; k < 2000; k += 2)
            if (!check(std::ldexp((double)k, -j), false)) return 1;
    const double specials[] = {0.0, 1.0, 255.0, 0.5, 1e-5, 1e-4, 9.999995e-5, 0.0001, 999999.4, 999999.5,
                               99999.95, 0.1, 1e-20, 5e-324, 2.2250738585072014e-308};
    for (double v : specials)
        if (!check(v, false)) return 1;
    printf("checked %ld values\n", checked);
    return 0;
}
