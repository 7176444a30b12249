// Checks the kernels' branch-free math (violet_gb300/csrc/vlt_math.cuh, host
// instantiation) against the oracle's piecewise restatement (oracle/omath.hpp) and
// the IEEE quotient, bit for bit:
//   exp2_ (select form) == orc::exp2_own;  exp2_fma (select) == exp2_fma_full
//   (piecewise, FMA Horner);  log2_ == orc::log2_own;  sincos_ == orc::sincos_own;
//   div_u8_255 / div_u12_4095 / div_u16_65535 == x / c for every x in [0, c].
// argv[1]: stride through the 2^32 binary32 bit patterns (1 = every value). Exit
// status 0 when nothing differs; the first mismatches are printed.
#include <stdio.h>
#include <stdlib.h>

#include "../../oracle/omath.hpp"
#include "../../violet_gb300/csrc/vlt_math.cuh"

static unsigned long long bad = 0;
static void report(const char* what, uint32_t u, uint32_t a, uint32_t b) {
  if (bad++ < 8) printf("%s 0x%08x: 0x%08x vs 0x%08x\n", what, u, a, b);
}

int main(int argc, char** argv) {
  const unsigned long long stride = argc > 1 ? strtoull(argv[1], nullptr, 10) : 1ull;
  unsigned long long n = 0;
  for (unsigned long long v = 0; v <= 0xFFFFFFFFull; v += stride) {
    const uint32_t u = (uint32_t)v;
    const float x = vlt::as_float(u);
    ++n;
    uint32_t a = vlt::as_uint(vlt::exp2_(x)), b = vlt::as_uint(orc::exp2_own(x));
    if (a != b) report("exp2", u, a, b);
    a = vlt::as_uint(vlt::exp2_fma(x));
    b = vlt::as_uint(vlt::exp2_fma_full(x));
    if (a != b) report("exp2_fma", u, a, b);
    a = vlt::as_uint(vlt::log2_(x));
    b = vlt::as_uint(orc::log2_own(x));
    if (a != b) report("log2", u, a, b);
    float s1, c1, s2, c2;
    vlt::sincos_(x, &s1, &c1);
    orc::sincos_own(x, &s2, &c2);
    if (vlt::as_uint(s1) != vlt::as_uint(s2)) report("sin", u, vlt::as_uint(s1), vlt::as_uint(s2));
    if (vlt::as_uint(c1) != vlt::as_uint(c2)) report("cos", u, vlt::as_uint(c1), vlt::as_uint(c2));
  }
  for (uint32_t x = 0; x <= 65535u; ++x) {
    volatile float f = (float)x;
    if (x <= 255u && vlt::as_uint(vlt::div_u8_255(x)) != vlt::as_uint(f / 255.0f))
      report("x/255", x, vlt::as_uint(vlt::div_u8_255(x)), vlt::as_uint(f / 255.0f));
    if (x <= 4095u && vlt::as_uint(vlt::div_u12_4095(x)) != vlt::as_uint(f / 4095.0f))
      report("x/4095", x, vlt::as_uint(vlt::div_u12_4095(x)), vlt::as_uint(f / 4095.0f));
    if (vlt::as_uint(vlt::div_u16_65535(x)) != vlt::as_uint(f / 65535.0f))
      report("x/65535", x, vlt::as_uint(vlt::div_u16_65535(x)), vlt::as_uint(f / 65535.0f));
  }
  printf("%llu values, %llu mismatches\n", n, bad);
  return bad ? 1 : 0;
}
