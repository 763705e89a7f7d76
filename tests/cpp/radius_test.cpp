// Host check of cadr::sphere_radius (cadr_gb300/csrc/fp.cuh): the float-float
// fast path with its double fallback must equal the reference's double
// evaluation float(sqrt(double(x)) * double(r)) on every input.
// Usage: radius_test <samples> <seed>; prints "mismatches=<k> hard=<h>".
#include "../../cadr_gb300/csrc/fp.cuh"
#include <cstdio>
#include <cstdlib>
#include <cstdint>

static uint64_t sm(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main(int argc, char** argv)
{
    const uint64_t n = argc > 1 ? strtoull(argv[1], nullptr, 10) : 10000000ull;
    uint64_t st = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1ull;
    uint64_t bad = 0, hard = 0;
    for (uint64_t i = 0; i < n; i++) {
        const uint64_t a = sm(st), b = sm(st);
        // x: random mantissa, exponent spanning the fast range and beyond;
        // r: random mantissa with exponent in [-40, 40]; every 16th sample
        // uses the scene-like ranges x in [0.25, 4], r in [0.01, 100].
        uint32_t xb, rb;
        if ((i & 15u) == 0) {
            xb = (uint32_t)((125u + (a >> 60) % 4u) << 23) | (uint32_t)(a & 0x7fffffu);
            rb = (uint32_t)((120u + (b >> 59) % 14u) << 23) | (uint32_t)(b & 0x7fffffu);
        } else {
            xb = (uint32_t)((1u + (a >> 40) % 253u) << 23) | (uint32_t)(a & 0x7fffffu);
            rb = (uint32_t)((87u + (b >> 40) % 80u) << 23) | (uint32_t)(b & 0x7fffffu);
        }
        const float x = cadr::bitsf(xb), r = cadr::bitsf(rb);
        const float f = cadr::sphere_radius(x, r);
        const float g = cadr::radius_double(x, r);
        if (cadr::fbits(f) != cadr::fbits(g)) {
            if (bad < 10) printf("x=%a r=%a fast=%a ref=%a\n", x, r, f, g);
            bad++;
        }
        // count inputs whose float-only product differs (the double rounding matters)
        if (cadr::fbits(cadr::fmul(cadr::fsqrt(x), r)) != cadr::fbits(g)) hard++;
    }
    printf("samples=%llu mismatches=%llu float_only_differs=%llu\n", (unsigned long long)n,
           (unsigned long long)bad, (unsigned long long)hard);
    return bad ? 1 : 0;
}
