/* Exhaustive check of the child-bound identity the traversal kernels use:
 *
 *     fmaf((float)q, 2^(e-8), origin)  ==  origin + ldexpf((float)q, e - 8)
 *
 * bit for bit, for every 8-bit q, every int8 exponent e, and a set of origins
 * (random bit patterns of every magnitude, signed zeros, denormals, the
 * largest finite values, infinities, and origins that cancel q * 2^(e-8)
 * exactly or nearly).  The right-hand side is the reference's set_child_bounds
 * (vulkan_acceleration_structure_util.h:499-508).  NaN results count as equal
 * when both sides are NaN.  Prints the number of mismatches and exits 1 if
 * there are any.  Build: cc -O2 -ffp-contract=off dequant_fma.c -lm
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint32_t bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

static float from_bits(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint32_t next_u32(void) { /* xorshift64* */
  state ^= state >> 12;
  state ^= state << 25;
  state ^= state >> 27;
  return (uint32_t)((state * 0x2545F4914F6CDD1Dull) >> 32);
}

static unsigned long long checked = 0, mismatches = 0;

static void check(uint32_t q, int e, float origin) {
  const float s = ldexpf(1.0f, e - 8);
  const float ref = origin + ldexpf((float)q, e - 8);
  const float got = fmaf((float)q, s, origin);
  ++checked;
  if (isnan(ref) && isnan(got)) return;
  if (bits(ref) != bits(got)) {
    if (mismatches < 10)
      printf("mismatch q=%u e=%d origin=%a: ref %a got %a\n", q, e, (double)origin, (double)ref, (double)got);
    ++mismatches;
  }
}

int main(void) {
  enum { N_RANDOM = 768 };
  float origins[N_RANDOM + 16];
  int n = 0;
  const uint32_t fixed[] = {0x00000000u, 0x80000000u, 0x00000001u, 0x80000001u, 0x007fffffu, 0x00800000u,
                            0x7f7fffffu, 0xff7fffffu, 0x7f800000u, 0xff800000u, 0x3f800000u, 0xbf800000u};
  for (unsigned i = 0; i < sizeof(fixed) / sizeof(fixed[0]); ++i) origins[n++] = from_bits(fixed[i]);
  while (n < N_RANDOM + 12) {
    const float f = from_bits(next_u32());
    if (!isnan(f)) origins[n++] = f;
  }
  for (int e = -128; e <= 127; ++e) {
    for (uint32_t q = 0; q < 256; ++q) {
      for (int i = 0; i < n; ++i) check(q, e, origins[i]);
      /* origins that cancel the product exactly, and one ulp either side */
      const float p = ldexpf((float)q, e - 8);
      check(q, e, -p);
      check(q, e, nextafterf(-p, INFINITY));
      check(q, e, nextafterf(-p, -INFINITY));
      /* origins a few binades above and below the product */
      check(q, e, p * 3.0f + 1.0f);
      check(q, e, -p * 0.75f);
      check(q, e, -p * 1048576.0f);
    }
  }
  printf("checked %llu, mismatches %llu\n", checked, mismatches);
  return mismatches ? 1 : 0;
}
