// Host check of the float-float helpers in csrc/tpm_ff.cuh (the mixed path's
// Poisson refinement): compiled with g++ against a stand-in cuda_runtime.h
// that maps the bit-cast intrinsics to memcpy, with contraction off so that
// the error-free transformations see the same IEEE float rounding as on the
// device.  Prints "ok" or the first failure.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "tpm_ff.cuh"
#define TPM_HOST_CHECK
#include "tpm_index.cuh"

using namespace tpm;

static int fails = 0;
#define CHECK(c, ...)                         \
  do {                                        \
    if (!(c) && fails++ < 10) {               \
      std::printf("FAIL %s: ", #c);           \
      std::printf(__VA_ARGS__);               \
      std::printf("\n");                      \
    }                                         \
  } while (0)

static double pair_value(float2 p) { return (double)p.x + (double)p.y; }

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> mant(1.0, 2.0), unit(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-74, 127);
  // split: |x - (hi + lo)| <= 2^-48 |x|, hi is x truncated to 24 bits
  for (int n = 0; n < 2000000; ++n) {
    double x = std::ldexp(mant(rng), ex(rng)) * (rng() & 1 ? -1.0 : 1.0);
    float2 p = ff_from_double(x);
    double err = std::fabs(x - pair_value(p));
    CHECK(err <= std::ldexp(std::fabs(x), -48), "x=%.17g err=%.3g", x, err);
    uint64_t b;
    std::memcpy(&b, &x, 8);
    b &= ~((uint64_t(1) << 29) - 1);
    double xt;
    std::memcpy(&xt, &b, 8);
    CHECK((double)p.x == xt, "x=%.17g hi=%.9g", x, (double)p.x);
  }
  // special values
  float2 z = ff_from_double(0.0), nz = ff_from_double(-0.0);
  CHECK(z.x == 0.f && z.y == 0.f && !std::signbit(z.x), "zero");
  CHECK(nz.x == 0.f && std::signbit(nz.x), "negative zero");
  float2 t = ff_from_double(-1e-30);  // below 2^-74: lo dropped
  CHECK(std::fabs(-1e-30 - pair_value(t)) <= std::ldexp(1e-30, -23), "tiny %.9g", (double)t.x);
  float2 u = ff_from_double(1e-40);  // below 2^-126: flushed
  CHECK(u.x == 0.f && u.y == 0.f, "underflow");
  CHECK(std::isinf(ff_from_double(1e39).x) && ff_from_double(1e39).x > 0, "overflow");
  CHECK(std::isinf(ff_from_double(-INFINITY).x) && ff_from_double(-INFINITY).x < 0, "-inf");
  CHECK(std::isnan(ff_from_double(NAN).x), "nan");
  // float -> double, exact
  std::uniform_int_distribution<uint32_t> bits;
  for (int n = 0; n < 2000000; ++n) {
    uint32_t w = bits(rng);
    float f;
    std::memcpy(&f, &w, 4);
    double d = ff_f2d(f);
    const uint32_t ef = (w >> 23) & 0xffu;
    if (ef == 0u)
      CHECK(d == 0.0 && std::signbit(d) == std::signbit(f), "subnormal/zero %08x", w);
    else if (std::isnan(f))
      CHECK(std::isnan(d), "nan %08x", w);
    else
      CHECK(d == (double)f, "f2d %08x", w);
  }
  // TwoSum is exact; the product stays within 2^-45, the sloppy add within 2^-46
  for (int n = 0; n < 2000000; ++n) {
    float a = (float)(unit(rng) * std::ldexp(1.0, ex(rng) / 8));
    float c = (float)(unit(rng) * std::ldexp(1.0, ex(rng) / 8));
    float2 s = ff_two_sum(a, c);
    CHECK((long double)s.x + s.y == (long double)a + c, "two_sum %.9g %.9g", a, c);
    float2 pa = ff_from_double(unit(rng) * 3.0), pb = ff_from_double(unit(rng) * 1e3);
    long double va = (long double)pa.x + pa.y, vb = (long double)pb.x + pb.y;
    float2 m = ff_mul(pa, pb);
    long double em = std::fabs((long double)m.x + m.y - va * vb);
    CHECK(em <= std::ldexp((long double)std::fabs(va * vb), -45), "mul err %.3Lg", em);
    float2 pc = ff_from_double(va * (1.0 + 1e-3 * unit(rng)));  // close to pa
    float2 sb = ff_sub(pc, pa);
    long double es = std::fabs((long double)sb.x + sb.y - (((long double)pc.x + pc.y) - va));
    CHECK(es <= std::ldexp(std::fabs(((long double)pc.x + pc.y) - va), -46), "sub err %.3Lg", es);
    float2 ss = ff_sub_sloppy(pa, pb);
    long double e2 = std::fabs((long double)ss.x + ss.y - (va - vb));
    CHECK(e2 <= std::ldexp(std::fabs(va) + std::fabs(vb), -46), "sloppy sub err %.3Lg", e2);
    float2 af = ff_add_f(pa, c);
    long double ef = std::fabs((long double)af.x + af.y - (va + c));
    CHECK(ef <= std::ldexp(std::fabs(va) + std::fabs((long double)c), -46), "add_f err %.3Lg", ef);
    float2 ad = ff_add(pa, pb);
    long double ea = std::fabs((long double)ad.x + ad.y - (va + vb));
    CHECK(ea <= std::ldexp(std::fabs(va) + std::fabs(vb), -46), "add err %.3Lg", ea);
  }
  // reciprocal of a split double and of a sum of two splits: within 2^-45
  for (int n = 0; n < 2000000; ++n) {
    const double x = std::ldexp(mant(rng), (int)(rng() % 200) - 100) * (rng() & 1 ? -1.0 : 1.0);
    const float2 r = ff_rcp(ff_from_double(x));
    const long double vx = pair_value(ff_from_double(x));
    const long double er = std::fabs(((long double)r.x + r.y) * vx - 1.0L);
    CHECK(er <= std::ldexp(1.0L, -45), "rcp x=%.17g err=%.3Lg", x, er);
    const double a = mant(rng), b = mant(rng) * std::ldexp(1.0, (int)(rng() % 5) - 2);
    const float2 s = ff_add(ff_from_double(a), ff_from_double(b));
    const float2 h = ff_rcp(s);
    const long double vs = (long double)s.x + s.y;
    const long double eh = std::fabs(((long double)h.x + h.y) * vs - 1.0L);
    CHECK(eh <= std::ldexp(1.0L, -45), "rcp of sum %.17g %.17g err=%.3Lg", a, b, eh);
  }
  // trunc / fraction / half decision from the bits of a double
  for (int n = 0; n < 2000000; ++n) {
    const double u = (rng() & 1 ? -1.0 : 1.0) *
                     std::ldexp(mant(rng), (int)(rng() % 40) - 20);  // 2^-20 .. 2^20
    int ip;
    float fr;
    bool up;
    ff_int_frac(u, ip, fr, up);
    const double t = std::trunc(u), f = u - t;  // exact
    CHECK(ip == (int)t, "trunc %.17g -> %d", u, ip);
    CHECK(std::fabs((double)fr - f) <= std::ldexp(std::fabs(f), -23) && std::fabs((double)fr) <= std::fabs(f),
          "frac %.17g -> %.9g", u, (double)fr);
    CHECK(up == (std::fabs(f) >= 0.5), "half %.17g", u);
  }
  for (double u : {0.0, 0.5, 1.0, 2.5, -2.5, 3.0, -0.25, 255.99999999999997}) {
    int ip;
    float fr;
    bool up;
    ff_int_frac(u, ip, fr, up);
    const double t = std::trunc(u), f = u - t;
    CHECK(ip == (int)t && std::fabs((double)fr) <= std::fabs(f) &&
              std::fabs((double)fr - f) <= std::ldexp(std::fabs(f), -23) &&
              up == (std::fabs(f) >= 0.5),
          "edge %.17g -> %d %.9g %d", u, ip, (double)fr, (int)up);
  }
  // trunc and the fraction as a pair: within 2^(e-48) of the exact fraction
  for (int n = 0; n < 2000000; ++n) {
    const double u = (rng() & 1 ? -1.0 : 1.0) *
                     std::ldexp(mant(rng), (int)(rng() % 40) - 20);  // 2^-20 .. 2^20
    int ip;
    float2 fr;
    ff_int_frac2(u, ip, fr);
    const double t = std::trunc(u), f = u - t;
    const int e = std::ilogb(u);
    CHECK(ip == (int)t, "trunc2 %.17g -> %d", u, ip);
    const long double ef = std::fabs((long double)fr.x + fr.y - f);
    CHECK(ef <= std::ldexp(1.0L, (e < 0 ? 0 : e) - 48) &&
              (e >= 0 || ef <= std::ldexp(std::fabs(u), -48)),
          "frac2 %.17g err %.3Lg", u, ef);
    CHECK(std::fabs(fr.y) <= std::ldexp(std::fabs(fr.x), -23), "frac2 normalised %.17g", u);
  }
  for (double u : {0.0, 0.5, 1.0, 2.5, -2.5, 3.0, -0.25, 255.99999999999997, 127.0 + 1e-13}) {
    int ip;
    float2 fr;
    ff_int_frac2(u, ip, fr);
    const double t = std::trunc(u), f = u - t;
    CHECK(ip == (int)t && std::fabs((long double)fr.x + fr.y - f) <= std::ldexp(1.0L, -40),
          "edge2 %.17g -> %d %.9g %.9g", u, ip, (double)fr.x, (double)fr.y);
  }
  // index division: every divisor up to 4096 against edge and random
  // numerators below 2^31
  for (unsigned d = 1; d <= 4096; ++d) {
    const unsigned long long m = udiv_magic(d);
    const unsigned edges[] = {0u, 1u, d - 1u, d, d + 1u, 2u * d - 1u, 0x7ffffffeu,
                              0x7fffffffu, (0x7fffffffu / d) * d, (0x7fffffffu / d) * d - 1u};
    for (unsigned a : edges) CHECK(udiv(a, m) == a / d, "udiv %u / %u", a, d);
    for (int n = 0; n < 2000; ++n) {
      const unsigned a = (unsigned)(rng() & 0x7fffffffu);
      CHECK(udiv(a, m) == a / d, "udiv %u / %u", a, d);
    }
  }
  for (unsigned d : {3u, 7u, 256u, 1000u, 2048u, 65535u, 65536u}) {
    const unsigned long long m = udiv_magic(d);
    for (unsigned a : {0xffffffffu, 0xfffffffeu, 0x80000000u})
      CHECK(udiv(a, m) == a / d, "udiv %u / %u", a, d);
  }
  if (fails) {
    std::printf("%d failures\n", fails);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
