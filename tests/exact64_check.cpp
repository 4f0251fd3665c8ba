// Host check of the integer-pipe FP64 square root and division
// (mps_gb300/csrc/exact64.cuh) against the host's IEEE operations, which
// round correctly.  The FP32 approximations the routines start from are
// perturbed by up to 2^-12 (the routines refine them by one Newton step; the
// hardware's documented bound is 2 ulp, about 2^-22), so the error budget
// itself is what is tested, not one particular approximation.
//
// usage: exact64_check <cases per family> <seed>; prints one line per family
// and exits 1 on the first mismatch.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../mps_gb300/csrc/exact64.cuh"

namespace {

std::mt19937_64 rng;
int mode = 0;  // 0: correctly rounded approximations, 1: random error, 2: +2^-12, 3: -2^-12

float perturb(double exact) {
    double u = 0.0;
    if (mode == 1) u = std::ldexp((double)(int64_t)(rng() >> 11) / 4503599627370496.0 - 1.0, -12);
    if (mode == 2) u = std::ldexp(1.0, -12);
    if (mode == 3) u = -std::ldexp(1.0, -12);
    return (float)(exact * (1.0 + u));
}

struct Approx {
    static float rsqrt(float x) { return perturb(1.0 / std::sqrt((double)x)); }
    static float rcp(float x) { return perturb(1.0 / (double)x); }
};

double from_parts(uint64_t mant, int biased_exp) {
    return mpsg::x64::double_of(((uint64_t)biased_exp << 52) | (mant & mpsg::x64::kMant));
}

uint64_t rand_mant() {
    const uint64_t r = rng();
    switch (r & 7) {
        case 0: return (r >> 8) & 0xff;                            // just above 2^52
        case 1: return mpsg::x64::kMant - ((r >> 8) & 0xff);       // just below 2^53
        case 2: return ((r >> 8) & 0xffff) << 36;                  // few low bits
        default: return r >> 12;
    }
}

bool same(double a, double b) { return mpsg::x64::bits_of(a) == mpsg::x64::bits_of(b); }

int check_sqrt(long n) {
    for (long i = 0; i < n; i++) {
        double x;
        if (i < 64) {  // the significands whose roots lie next to a midpoint
            const uint64_t tbl[4] = {1, mpsg::x64::kMant, 0, mpsg::x64::kMant - 1};
            x = from_parts(tbl[i & 3], 1 + (int)((i >> 2) * 127 % 2046));
        } else {
            x = from_parts(rand_mant(), 1 + (int)(rng() % 2046));
        }
        double got;
        if (!mpsg::x64::sqrt_rn<Approx>(x, got)) {
            std::printf("sqrt: fast path refused %a\n", x);
            return 1;
        }
        const double want = std::sqrt(x);
        if (!same(got, want)) {
            std::printf("sqrt mismatch (mode %d): x=%a got %a want %a\n", mode, x, got, want);
            return 1;
        }
    }
    return 0;
}

int check_div(long n) {
    long refused = 0;
    for (long i = 0; i < n; i++) {
        const int ea = 1 + (int)(rng() % 2046);
        int eb = ea + (int)(rng() % 201) - 100;
        if (eb < 1) eb = 1;
        if (eb > 2046) eb = 2046;
        uint64_t ma = rand_mant(), mb = rand_mant();
        if ((i & 15) == 0) mb = ma;                                 // equal significands
        if ((i & 15) == 1) mb = ma + 1 <= mpsg::x64::kMant ? ma + 1 : ma - 1;
        double a = from_parts(ma, ea), b = from_parts(mb, eb);
        if (rng() & 1) a = -a;
        if (rng() & 1) b = -b;
        double got;
        const double want = a / b;
        if (!mpsg::x64::div_rn<Approx>(a, b, got)) {
            // refused only where the rounded significand's binade leaves the
            // normal range (a result of 2^-1022 may come from a subnormal one
            // rounding up)
            const double aw = std::fabs(want);
            if (aw >= 0x1p-1021 && aw < 0x1p1023) {
                std::printf("div: fast path refused %a / %a\n", a, b);
                return 1;
            }
            refused++;
            continue;
        }
        if (!same(got, want)) {
            std::printf("div mismatch (mode %d): %a / %a got %a want %a\n", mode, a, b, got, want);
            return 1;
        }
    }
    return 0;
}

int check_refusals() {
    double out;
    const double bad[] = {0.0, -0.0, -1.0, 0x1p-1074, 0x1p-1030, INFINITY, NAN};
    for (double x : bad)
        if (mpsg::x64::sqrt_rn<Approx>(x, out)) {
            std::printf("sqrt: fast path taken for %a\n", x);
            return 1;
        }
    const double pairs[][2] = {{1.0, 0.0}, {0.0, 1.0}, {INFINITY, 1.0}, {1.0, NAN}, {0x1p1000, 0x1p-100},
                               {0x1p-1000, 0x1p100}, {0x1p-1060, 1.0}};
    for (auto& p : pairs)
        if (mpsg::x64::div_rn<Approx>(p[0], p[1], out)) {
            std::printf("div: fast path taken for %a / %a\n", p[0], p[1]);
            return 1;
        }
    return 0;
}

int check_small_ops(long n) {
    for (long i = 0; i < n; i++) {
        // q - 1 for q in [1, 2^53), every binade
        const double q = from_parts(rand_mant(), 1023 + (int)(rng() % 53));
        double got;
        if (!mpsg::x64::sub_one(q, got) || !same(got, q - 1.0)) {
            std::printf("sub_one mismatch: %a\n", q);
            return 1;
        }
        // FP32 rounding of doubles around and inside the FP32 range
        double x = from_parts(rand_mant(), 880 + (int)(rng() % 290));
        if (rng() & 1) x = -x;
        float f;
        if (mpsg::x64::to_f32(x, f)) {
            if (mpsg::x64::u_of(f) != mpsg::x64::u_of((float)x)) {
                std::printf("to_f32 mismatch: %a\n", x);
                return 1;
            }
        } else if (std::fabs(x) >= 0x1p-126 && std::isfinite((float)x)) {
            std::printf("to_f32 refused %a\n", x);
            return 1;
        }
        // the ordering shortcut on non-negative values
        const double v = from_parts(rand_mant(), 1000 + (int)(rng() % 40));
        const double cut = from_parts(rand_mant(), 1000 + (int)(rng() % 40));
        if (mpsg::x64::lt_cut(v, cut) != (v < cut) || mpsg::x64::lt_cut(cut, cut)) {
            std::printf("lt_cut mismatch: %a %a\n", v, cut);
            return 1;
        }
    }
    double out;
    float fo;
    if (mpsg::x64::sub_one(0.5, out) || mpsg::x64::sub_one(0x1p53, out) || mpsg::x64::sub_one(INFINITY, out) ||
        !mpsg::x64::sub_one(1.0, out) || out != 0.0 || std::signbit(out) ||
        !mpsg::x64::to_f32(-0.0, fo) || !std::signbit(fo) || mpsg::x64::to_f32(1e-300, fo) ||
        mpsg::x64::to_f32(NAN, fo) || !mpsg::x64::lt_cut(0.0, 1.0) || mpsg::x64::lt_cut(NAN, 1.0) ||
        mpsg::x64::lt_cut(INFINITY, 1.0)) {
        std::printf("small ops: special case wrong\n");
        return 1;
    }
    std::printf("%ld subtractions of one, FP32 roundings and comparisons bit-identical\n", n);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    rng.seed(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1);
    if (check_refusals() || check_small_ops(n)) return 1;
    for (mode = 0; mode < 4; mode++) {
        if (check_sqrt(n) || check_div(n)) return 1;
        std::printf("mode %d: %ld square roots and %ld quotients bit-identical\n", mode, n, n);
    }
    return 0;
}
