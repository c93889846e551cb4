// Compares the runtime's printf formatter (csrc/fmt.h, compiled for the host)
// with the host C library's snprintf on seeded random values and conversion
// specifications.  Prints one line per mismatch and a final count; exit status
// is 0 only when every case matches byte for byte.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "fmt.h"

static uint64_t sm_state;
static uint64_t next_u64() {  // splitmix64
    uint64_t z = (sm_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static double random_double() {
    uint64_t k = next_u64() % 10;
    if (k < 4) {  // any bit pattern (subnormals, huge, inf, nan included)
        uint64_t b = next_u64();
        double d;
        memcpy(&d, &b, 8);
        return d;
    }
    if (k < 8) {  // moderate magnitudes where rounding decisions matter
        double m = (double)(next_u64() >> 11) / 9007199254740992.0;
        int e = (int)(next_u64() % 60) - 30;
        return (next_u64() & 1 ? -1 : 1) * ldexp(m, e) * pow(10.0, (int)(next_u64() % 9) - 4);
    }
    static const double special[] = {0.0, -0.0, 0.5, 1.5, 2.5, 0.125, 1e-320, 1e308, 123456789.0, 0.1, 9.5,
                                     99.995, 0.000049999, 1e22, 5e-324};
    return special[next_u64() % (sizeof(special) / sizeof(special[0]))];
}

static int fails = 0, cases = 0;

static void check(const char* spec, const char* a, const char* b, int na, int nb) {
    cases++;
    if (na != nb || strcmp(a, b) != 0) {
        if (fails < 40) printf("MISMATCH spec=%s ours=[%s](%d) libc=[%s](%d)\n", spec, a, na, b, nb);
        fails++;
    }
}

int main(int argc, char** argv) {
    long iters = argc > 1 ? atol(argv[1]) : 20000;
    sm_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 12345;
    static const char flagset[][6] = {"", "-", "+", " ", "#", "0", "-+", "+0", "#0", " 0", "-#", "+#0"};
    static const char fconv[] = "fFeEgGaA";
    static const char iconv[] = "diuoxX";
    char spec[64], a[2048], b[2048];
    for (long it = 0; it < iters; it++) {
        const char* fl = flagset[next_u64() % 12];
        int w = (int)(next_u64() % 4) == 0 ? -1 : (int)(next_u64() % 30);
        int p = (int)(next_u64() % 3) == 0 ? -1 : (int)(next_u64() % 40);
        char ws[16] = "", ps[16] = "";
        if (w >= 0) snprintf(ws, sizeof ws, "%d", w);
        if (p >= 0) snprintf(ps, sizeof ps, ".%d", p);
        // floating point
        double d = random_double();
        char c = fconv[next_u64() % 8];
        snprintf(spec, sizeof spec, "%%%s%s%s%c", fl, ws, ps, c);
        int na = gmfmt::format(a, sizeof a, spec, d);
        int nb = snprintf(b, sizeof b, spec, d);
        check(spec, a, b, na, nb);
        // integers with length modifiers
        char ic = iconv[next_u64() % 6];
        uint64_t v = next_u64() >> (next_u64() % 64);
        switch (next_u64() % 5) {
            case 0:
                snprintf(spec, sizeof spec, "%%%s%s%s%c", fl, ws, ps, ic);
                na = gmfmt::format(a, sizeof a, spec, (int)v);
                nb = snprintf(b, sizeof b, spec, (int)v);
                break;
            case 1:
                snprintf(spec, sizeof spec, "%%%s%s%sl%c", fl, ws, ps, ic);
                na = gmfmt::format(a, sizeof a, spec, (long)v);
                nb = snprintf(b, sizeof b, spec, (long)v);
                break;
            case 2:
                snprintf(spec, sizeof spec, "%%%s%s%sll%c", fl, ws, ps, ic);
                na = gmfmt::format(a, sizeof a, spec, (long long)v);
                nb = snprintf(b, sizeof b, spec, (long long)v);
                break;
            case 3:
                snprintf(spec, sizeof spec, "%%%s%s%sh%c", fl, ws, ps, ic);
                na = gmfmt::format(a, sizeof a, spec, (int)v);
                nb = snprintf(b, sizeof b, spec, (int)v);
                break;
            default:
                snprintf(spec, sizeof spec, "%%%s%s%shh%c", fl, ws, ps, ic);
                na = gmfmt::format(a, sizeof a, spec, (int)v);
                nb = snprintf(b, sizeof b, spec, (int)v);
                break;
        }
        check(spec, a, b, na, nb);
    }
    // strings, characters, pointers, star width/precision, literal text
    const char* s = "hello, world";
    static const char* sspec[] = {"%s|", "%20s|", "%-20s|", "%.5s|", "%8.3s|", "%-8.0s|", "[%c%c%c]", "%%|%5c|%-5c|"};
    for (const char* sp : sspec) {
        int na, nb;
        if (strchr(sp, 'c')) {
            na = gmfmt::format(a, sizeof a, sp, 'x', 'y', 'z');
            nb = snprintf(b, sizeof b, sp, 'x', 'y', 'z');
        } else {
            na = gmfmt::format(a, sizeof a, sp, s);
            nb = snprintf(b, sizeof b, sp, s);
        }
        check(sp, a, b, na, nb);
    }
    for (int w = -12; w <= 12; w += 3)
        for (int p = -1; p <= 9; p += 2) {
            int na = gmfmt::format(a, sizeof a, "<%*.*f|%*d|%.*s>", w, p, 3.14159265358979, w, 42, p, s);
            int nb = snprintf(b, sizeof b, "<%*.*f|%*d|%.*s>", w, p, 3.14159265358979, w, 42, p, s);
            check("star", a, b, na, nb);
        }
    void* ptrs[] = {nullptr, (void*)0x1234, (void*)0x7fffdeadbeefull};
    for (void* q : ptrs) {
        int na = gmfmt::format(a, sizeof a, "%p %20p %-20p|", q, q, q);
        int nb = snprintf(b, sizeof b, "%p %20p %-20p|", q, q, q);
        check("%p", a, b, na, nb);
    }
    // truncation: the return value counts the full output
    {
        char sa[8], sb[8];
        int na = gmfmt::format(sa, sizeof sa, "%s-%d-%.3e", s, 123456, 6.02214076e23);
        int nb = snprintf(sb, sizeof sb, "%s-%d-%.3e", s, 123456, 6.02214076e23);
        check("truncate", sa, sb, na, nb);
    }
    printf("fmt_check cases %d mismatches %d\n", cases, fails);
    return fails ? 1 : 0;
}
