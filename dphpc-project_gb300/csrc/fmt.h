// printf-family formatter shared by device code and host tests.
//
// Conversions: d i u o x X c s p n % and f F e E g G a A, with flags
// (- + space # 0), field width, precision ('*' allowed) and length modifiers
// (hh h l ll z j t L).  Floating-point conversions are exact: the decimal
// digits of the binary value are generated with multi-word integer arithmetic
// and rounded to nearest, ties to even, on the exact value, which is what
// glibc's printf does in the default rounding mode.  Output therefore matches
// the host C library byte for byte, so program output can be compared between
// a GPU run and a host MPI run.
#pragma once

#include <stdarg.h>
#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define GM_HD __host__ __device__
#define GM_NOINLINE __noinline__
#else
#define GM_HD
#define GM_NOINLINE __attribute__((noinline))
#endif

namespace gmfmt {

struct Sink {
    char* out;
    size_t cap;   // bytes available including the terminating NUL
    size_t len;   // characters produced so far (may exceed cap)
    GM_HD void put(char c) {
        if (len + 1 < cap) out[len] = c;
        len++;
    }
    GM_HD void rep(char c, int n) {
        for (int i = 0; i < n; i++) put(c);
    }
    GM_HD void str(const char* s, int n) {
        for (int i = 0; i < n; i++) put(s[i]);
    }
};

// Little-endian multi-word unsigned integer, enough for 2^1100.
struct Big {
    uint32_t d[40];
    int n;
    GM_HD void set_u64(uint64_t v) {
        n = 0;
        while (v) {
            d[n++] = (uint32_t)v;
            v >>= 32;
        }
    }
    GM_HD bool zero() const { return n == 0; }
    GM_HD void shl(int s) {
        if (n == 0 || s == 0) return;
        int w = s / 32, b = s % 32;
        int nn = n + w + 1;
        for (int i = nn - 1; i >= 0; i--) {
            uint64_t hi = (i - w >= 0 && i - w < n) ? d[i - w] : 0;
            uint64_t lo = (i - w - 1 >= 0 && i - w - 1 < n) ? d[i - w - 1] : 0;
            uint32_t v = b ? (uint32_t)((hi << b) | (lo >> (32 - b))) : (uint32_t)hi;
            d[i] = v;
        }
        n = nn;
        while (n > 0 && d[n - 1] == 0) n--;
    }
    GM_HD void mul_small(uint32_t m) {
        uint64_t carry = 0;
        for (int i = 0; i < n; i++) {
            uint64_t v = (uint64_t)d[i] * m + carry;
            d[i] = (uint32_t)v;
            carry = v >> 32;
        }
        if (carry) d[n++] = (uint32_t)carry;
    }
    // Divide in place by m, return the remainder.
    GM_HD uint32_t divmod_small(uint32_t m) {
        uint64_t rem = 0;
        for (int i = n - 1; i >= 0; i--) {
            uint64_t cur = (rem << 32) | d[i];
            d[i] = (uint32_t)(cur / m);
            rem = cur % m;
        }
        while (n > 0 && d[n - 1] == 0) n--;
        return (uint32_t)rem;
    }
    // Remove and return the bits at and above bit s (s >= 0); keeps bits below s.
    GM_HD uint32_t take_above(int s) {
        int w = s / 32, b = s % 32;
        uint64_t v = 0;
        for (int i = n - 1; i >= w; i--) {
            uint64_t limb = d[i];
            if (i == w) limb >>= b;
            v = (v << (i == w ? 32 - b : 32)) | limb;
        }
        if (w < n) {
            if (b == 0) {
                n = w;
            } else {
                d[w] &= (uint32_t)((1ull << b) - 1);
                n = w + 1;
            }
        }
        while (n > 0 && d[n - 1] == 0) n--;
        return (uint32_t)v;
    }
};

// Exact decimal digit stream of a finite, non-negative double.
struct Digits {
    char ip[330];   // integer part digits, most significant first
    int nip;        // 0 when the integer part is zero
    Big frac;       // fractional numerator over 2^fs
    int fs;
    GM_HD void init(double v) {
        uint64_t bits;
        memcpy_bits(&bits, &v);
        int ex = (int)((bits >> 52) & 0x7ff);
        uint64_t m = bits & ((1ull << 52) - 1);
        int e;
        if (ex == 0) {
            e = -1074;
        } else {
            m |= 1ull << 52;
            e = ex - 1075;
        }
        Big ib;
        if (e >= 0) {
            ib.set_u64(m);
            ib.shl(e);
            frac.n = 0;
            fs = 0;
        } else {
            fs = -e;
            if (fs >= 64) {
                ib.n = 0;
            } else {
                ib.set_u64(m >> fs);
            }
            uint64_t fm = fs >= 64 ? m : (m & ((1ull << fs) - 1));
            frac.set_u64(fm);
        }
        // integer part to decimal
        char tmp[330];
        int nt = 0;
        while (!ib.zero()) {
            uint32_t r = ib.divmod_small(1000000000u);
            for (int k = 0; k < 9; k++) {
                tmp[nt++] = (char)('0' + r % 10);
                r /= 10;
            }
        }
        while (nt > 0 && tmp[nt - 1] == '0') nt--;
        nip = nt;
        for (int i = 0; i < nt; i++) ip[i] = tmp[nt - 1 - i];
    }
    static GM_HD void memcpy_bits(uint64_t* b, const double* v) {
        const unsigned char* s = (const unsigned char*)v;
        unsigned char* d = (unsigned char*)b;
        for (int i = 0; i < 8; i++) d[i] = s[i];
    }
    // next fractional digit
    GM_HD int next_frac() {
        if (frac.zero()) return 0;
        frac.mul_small(10);
        return (int)frac.take_above(fs);
    }
    GM_HD bool frac_zero() const { return frac.zero(); }
};

// Round a digit string up by one unit in its last place; returns 1 when a
// carry spills out of the first digit (the string is then all zeros).
static GM_HD int round_up(char* s, int n) {
    for (int i = n - 1; i >= 0; i--) {
        if (s[i] == '9') {
            s[i] = '0';
        } else {
            s[i]++;
            return 0;
        }
    }
    return 1;
}

static GM_HD bool should_round_up(int next, bool sticky, char last) {
    if (next > 5) return true;
    if (next < 5) return false;
    if (sticky) return true;
    return ((last - '0') & 1) != 0;
}

struct Spec {
    bool left, plus, space, alt, zero;
    int width;
    int prec;   // -1 = default
    char conv;
};

static GM_HD void pad_out(Sink& o, const Spec& sp, const char* sign, int nsign, const char* body,
                          int nbody, const char* prefix = "", int nprefix = 0, int zeros = 0) {
    int total = nsign + nprefix + zeros + nbody;
    int padn = sp.width > total ? sp.width - total : 0;
    if (!sp.left && !sp.zero) o.rep(' ', padn);
    o.str(sign, nsign);
    o.str(prefix, nprefix);
    if (!sp.left && sp.zero) o.rep('0', padn);
    o.rep('0', zeros);
    o.str(body, nbody);
    if (sp.left) o.rep(' ', padn);
}

// Significant digits with decimal exponent: value = 0.d1d2... * 10^(E+1).
// Produces `nsig` rounded significant digits into sig and returns E.
static GM_HD GM_NOINLINE int sig_digits(double v, int nsig, char* sig, bool* carried = nullptr) {
    if (carried) *carried = false;
    Digits dg;
    dg.init(v);
    int E;
    int k = 0;
    int next = 0;
    bool sticky = false;
    if (dg.nip > 0) {
        E = dg.nip - 1;
        int i = 0;
        for (; i < dg.nip && k < nsig; i++) sig[k++] = dg.ip[i];
        if (k < nsig) {
            while (k < nsig) sig[k++] = (char)('0' + dg.next_frac());
            next = dg.next_frac();
            sticky = !dg.frac_zero();
        } else {
            if (i < dg.nip) {
                next = dg.ip[i++] - '0';
                for (; i < dg.nip; i++)
                    if (dg.ip[i] != '0') sticky = true;
                if (!dg.frac_zero()) sticky = true;
            } else {
                next = dg.next_frac();
                sticky = !dg.frac_zero();
            }
        }
    } else {
        E = -1;
        int d = dg.next_frac();
        while (d == 0) {
            E--;
            d = dg.next_frac();
        }
        sig[k++] = (char)('0' + d);
        while (k < nsig) sig[k++] = (char)('0' + dg.next_frac());
        next = dg.next_frac();
        sticky = !dg.frac_zero();
    }
    if (should_round_up(next, sticky, sig[nsig - 1])) {
        if (round_up(sig, nsig)) {
            sig[0] = '1';
            for (int i = 1; i < nsig; i++) sig[i] = '0';
            E++;
            if (carried) *carried = true;
        }
    }
    return E;
}

static GM_HD int fmt_exp(char* b, int E, bool upper) {
    int n = 0;
    b[n++] = upper ? 'E' : 'e';
    b[n++] = E < 0 ? '-' : '+';
    int a = E < 0 ? -E : E;
    char t[8];
    int nt = 0;
    do {
        t[nt++] = (char)('0' + a % 10);
        a /= 10;
    } while (a);
    if (nt < 2) t[nt++] = '0';
    for (int i = nt - 1; i >= 0; i--) b[n++] = t[i];
    return n;
}

static GM_HD GM_NOINLINE void fmt_float(Sink& o, Spec sp, double v) {
    uint64_t bits;
    Digits::memcpy_bits(&bits, &v);
    const bool neg = (bits >> 63) != 0;
    const bool upper = sp.conv == 'F' || sp.conv == 'E' || sp.conv == 'G' || sp.conv == 'A';
    char sign[1];
    int nsign = 0;
    if (neg) sign[nsign++] = '-';
    else if (sp.plus) sign[nsign++] = '+';
    else if (sp.space) sign[nsign++] = ' ';
    const int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0x7ff) {
        const bool nan = (bits & ((1ull << 52) - 1)) != 0;
        const char* s = nan ? (upper ? "NAN" : "nan") : (upper ? "INF" : "inf");
        sp.zero = false;
        pad_out(o, sp, sign, nsign, s, 3);
        return;
    }
    double a = neg ? -v : v;
    char body[1500];
    int nb = 0;
    char c = sp.conv;
    if (c == 'a' || c == 'A') {
        // hexadecimal: [-]0xh.hhhp[+-]d, shortest exact unless a precision is given
        uint64_t m = bits & ((1ull << 52) - 1);
        int e = ex == 0 ? (m ? -1022 : 0) : ex - 1023;
        int lead = ex == 0 ? 0 : 1;
        int prec = sp.prec;
        if (prec >= 0 && prec < 13) {
            int drop = (13 - prec) * 4;
            uint64_t full = ((uint64_t)lead << 52) | m;
            uint64_t rem = full & ((1ull << drop) - 1);
            uint64_t half = 1ull << (drop - 1);
            full >>= drop;
            if (rem > half || (rem == half && (full & 1))) full++;
            lead = (int)(full >> (prec * 4));
            m = (full & ((prec ? (1ull << (prec * 4)) : 1) - 1)) << drop;
            if (prec == 0) m = 0;
        }
        const char* hx = upper ? "0123456789ABCDEF" : "0123456789abcdef";
        body[nb++] = (char)('0' + lead);
        int nd = 13;
        if (prec < 0) {
            while (nd > 0 && ((m >> ((13 - nd) * 4)) & 0xf) == 0) nd--;
        } else {
            nd = prec < 13 ? prec : 13;
        }
        if (nd > 0 || sp.alt) body[nb++] = '.';
        for (int i = 0; i < nd; i++) body[nb++] = hx[(m >> ((12 - i) * 4)) & 0xf];
        if (prec > 13)
            for (int i = 13; i < prec; i++) body[nb++] = '0';
        body[nb++] = upper ? 'P' : 'p';
        body[nb++] = e < 0 ? '-' : '+';
        int ae = e < 0 ? -e : e;
        char t[8];
        int nt = 0;
        do {
            t[nt++] = (char)('0' + ae % 10);
            ae /= 10;
        } while (ae);
        for (int i = nt - 1; i >= 0; i--) body[nb++] = t[i];
        pad_out(o, sp, sign, nsign, body, nb, upper ? "0X" : "0x", 2);
        return;
    }
    int prec = sp.prec < 0 ? 6 : sp.prec;
    if (prec > 700) prec = 700;
    if (c == 'g' || c == 'G') {
        int P = prec == 0 ? 1 : prec;
        char sig[720];
        int E = 0;
        bool carried = false;
        if (a == 0.0) {
            for (int i = 0; i < P; i++) sig[i] = '0';
            E = 0;
        } else {
            E = sig_digits(a, P, sig, &carried);
        }
        // glibc picks the style from the exponent before rounding: a value
        // just below 10^P that rounds up to it was set for fixed style with no
        // fraction digits, and glibc keeps that digit count when it switches
        // to exponent style ("%#.2g" of 99.96 prints "1.e+02").
        const bool glibc_carry = sp.alt && carried && E == P;
        int nsig = P;
        if (!sp.alt)
            while (nsig > 1 && sig[nsig - 1] == '0') nsig--;
        if (P > E && E >= -4) {
            // fixed style with P-1-E fraction digits (before trailing-zero removal)
            if (E >= 0) {
                for (int i = 0; i <= E; i++) body[nb++] = i < nsig ? sig[i] : '0';
                int nf = sp.alt ? P - 1 - E : nsig - 1 - E;
                if (nf > 0 || sp.alt) body[nb++] = '.';
                for (int i = 0; i < nf; i++) body[nb++] = (E + 1 + i) < nsig ? sig[E + 1 + i] : '0';
            } else {
                body[nb++] = '0';
                int nf = sp.alt ? P - 1 - E : nsig - 1 - E;
                body[nb++] = '.';
                for (int i = 0; i < -E - 1; i++) body[nb++] = '0';
                for (int i = 0; i < nf + E + 1; i++) body[nb++] = sig[i];
            }
        } else {
            body[nb++] = sig[0];
            int nf = glibc_carry ? 0 : sp.alt ? P - 1 : nsig - 1;
            if (nf > 0 || sp.alt) body[nb++] = '.';
            for (int i = 1; i <= nf; i++) body[nb++] = sig[i];
            nb += fmt_exp(body + nb, E, upper);
        }
        pad_out(o, sp, sign, nsign, body, nb);
        return;
    }
    if (c == 'e' || c == 'E') {
        char sig[720];
        int E = 0;
        if (a == 0.0) {
            for (int i = 0; i <= prec; i++) sig[i] = '0';
        } else {
            E = sig_digits(a, prec + 1, sig);
        }
        body[nb++] = sig[0];
        if (prec > 0 || sp.alt) body[nb++] = '.';
        for (int i = 1; i <= prec; i++) body[nb++] = sig[i];
        nb += fmt_exp(body + nb, E, upper);
        pad_out(o, sp, sign, nsign, body, nb);
        return;
    }
    // fixed
    {
        Digits dg;
        dg.init(a);
        char ds[1100];
        int nd = 0;
        if (dg.nip == 0) ds[nd++] = '0';
        for (int i = 0; i < dg.nip; i++) ds[nd++] = dg.ip[i];
        const int nint = nd;
        for (int i = 0; i < prec; i++) ds[nd++] = (char)('0' + dg.next_frac());
        int next = dg.next_frac();
        bool sticky = !dg.frac_zero();
        int carry = 0;
        if (should_round_up(next, sticky, ds[nd - 1])) carry = round_up(ds, nd);
        if (carry) body[nb++] = '1';
        for (int i = 0; i < nint; i++) body[nb++] = ds[i];
        if (prec > 0 || sp.alt) body[nb++] = '.';
        for (int i = nint; i < nd; i++) body[nb++] = ds[i];
        pad_out(o, sp, sign, nsign, body, nb);
    }
}

static GM_HD GM_NOINLINE void fmt_int(Sink& o, Spec sp, unsigned long long u, bool neg) {
    char buf[72];
    int n = 0;
    int base = 10;
    const char* dig = "0123456789abcdef";
    if (sp.conv == 'x') base = 16;
    if (sp.conv == 'X') {
        base = 16;
        dig = "0123456789ABCDEF";
    }
    if (sp.conv == 'o') base = 8;
    unsigned long long t = u;
    while (t) {
        buf[n++] = dig[t % base];
        t /= base;
    }
    char body[72];
    int nb = 0;
    for (int i = n - 1; i >= 0; i--) body[nb++] = buf[i];
    int zeros = 0;
    if (sp.prec >= 0) {
        if (nb < sp.prec) zeros = sp.prec - nb;
        sp.zero = false;
    } else if (nb == 0) {
        zeros = 1;
    }
    if (sp.conv == 'o' && sp.alt && zeros == 0 && (nb == 0 || body[0] != '0')) zeros = 1;
    char sign[1];
    int nsign = 0;
    if (sp.conv == 'd' || sp.conv == 'i') {
        if (neg) sign[nsign++] = '-';
        else if (sp.plus) sign[nsign++] = '+';
        else if (sp.space) sign[nsign++] = ' ';
    }
    const char* prefix = "";
    int np = 0;
    if (sp.alt && u != 0 && base == 16) {
        prefix = sp.conv == 'X' ? "0X" : "0x";
        np = 2;
    }
    pad_out(o, sp, sign, nsign, body, nb, prefix, np, zeros);
}

// vsnprintf semantics.
static GM_HD GM_NOINLINE int vformat(char* out, size_t cap, const char* f, va_list ap) {
    Sink o;
    o.out = out;
    o.cap = cap;
    o.len = 0;
    while (*f) {
        if (*f != '%') {
            o.put(*f++);
            continue;
        }
        f++;
        if (*f == '%') {
            o.put('%');
            f++;
            continue;
        }
        Spec sp;
        sp.left = sp.plus = sp.space = sp.alt = sp.zero = false;
        sp.width = 0;
        sp.prec = -1;
        for (;; f++) {
            if (*f == '-') sp.left = true;
            else if (*f == '+') sp.plus = true;
            else if (*f == ' ') sp.space = true;
            else if (*f == '#') sp.alt = true;
            else if (*f == '0') sp.zero = true;
            else break;
        }
        if (*f == '*') {
            int w = va_arg(ap, int);
            if (w < 0) {
                sp.left = true;
                w = -w;
            }
            sp.width = w;
            f++;
        } else {
            while (*f >= '0' && *f <= '9') sp.width = sp.width * 10 + (*f++ - '0');
        }
        if (*f == '.') {
            f++;
            sp.prec = 0;
            if (*f == '*') {
                int p = va_arg(ap, int);
                sp.prec = p < 0 ? -1 : p;
                f++;
            } else {
                while (*f >= '0' && *f <= '9') sp.prec = sp.prec * 10 + (*f++ - '0');
            }
        }
        if (sp.left) sp.zero = false;
        int len = 0;  // 1 hh, 2 h, 3 l, 4 ll, 5 z/j/t, 6 L
        if (*f == 'h') {
            f++;
            len = 2;
            if (*f == 'h') {
                f++;
                len = 1;
            }
        } else if (*f == 'l') {
            f++;
            len = 3;
            if (*f == 'l') {
                f++;
                len = 4;
            }
        } else if (*f == 'z' || *f == 'j' || *f == 't') {
            f++;
            len = 5;
        } else if (*f == 'L') {
            f++;
            len = 6;
        }
        sp.conv = *f;
        if (!*f) break;
        f++;
        switch (sp.conv) {
            case 'd':
            case 'i': {
                long long v;
                if (len >= 3) v = va_arg(ap, long long);
                else v = va_arg(ap, int);
                if (len == 1) v = (signed char)v;
                if (len == 2) v = (short)v;
                unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
                fmt_int(o, sp, u, v < 0);
                break;
            }
            case 'u':
            case 'x':
            case 'X':
            case 'o': {
                unsigned long long u;
                if (len >= 3) u = va_arg(ap, unsigned long long);
                else u = va_arg(ap, unsigned int);
                if (len == 1) u = (unsigned char)u;
                if (len == 2) u = (unsigned short)u;
                fmt_int(o, sp, u, false);
                break;
            }
            case 'c': {
                char ch = (char)va_arg(ap, int);
                sp.zero = false;
                pad_out(o, sp, "", 0, &ch, 1);
                break;
            }
            case 's': {
                const char* s = va_arg(ap, const char*);
                if (!s) s = "(null)";
                int n = 0;
                while (s[n] && (sp.prec < 0 || n < sp.prec)) n++;
                sp.zero = false;
                pad_out(o, sp, "", 0, s, n);
                break;
            }
            case 'p': {
                void* p = va_arg(ap, void*);
                sp.zero = false;
                if (!p) {
                    pad_out(o, sp, "", 0, "(nil)", 5);
                } else {
                    Spec h = sp;
                    h.conv = 'x';
                    h.alt = true;
                    fmt_int(o, h, (unsigned long long)(uintptr_t)p, false);
                }
                break;
            }
            case 'n': {
                int* p = va_arg(ap, int*);
                if (p) *p = (int)o.len;
                break;
            }
            case 'f':
            case 'F':
            case 'e':
            case 'E':
            case 'g':
            case 'G':
            case 'a':
            case 'A': {
                double v = va_arg(ap, double);
                fmt_float(o, sp, v);
                break;
            }
            default:
                o.put('%');
                o.put(sp.conv);
                break;
        }
    }
    if (cap > 0) o.out[o.len < cap ? o.len : cap - 1] = 0;
    return (int)o.len;
}

static GM_HD int format(char* out, size_t cap, const char* f, ...) {
    va_list ap;
    va_start(ap, f);
    int n = vformat(out, cap, f, ap);
    va_end(ap);
    return n;
}

}  // namespace gmfmt
