// Host check of the certified float-float bicubic (csrc/bp_cubic.h) against
// the reference's double expression (WaP_Tomo.cpp:208-222, 1618): whenever
// cubic_cert / update_cert claim a result, it must equal the double
// expression rounded to float, bit for bit.  The same for grow_cert against
// CImg's cubic growth in double (CImg.h:28432-28610) with random double
// weights t, t*t, (t*t)*t.  Inputs: correction-image-like
// values of many magnitudes, exact ties and cancellations, random bit
// patterns, and the interpolation weights the backprojection produces
// (multiples of 2^-22 in [0, 1)).  Prints counts; exits 1 on any mismatch.
//
//   g++ -O2 -std=c++17 -ffp-contract=off -I<csrc> bp_cubic_check.cpp -o check && ./check [cases] [seed]
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bp_cubic.h"

static float cubic_double(float p0, float p1, float p2, float p3, float x) {
  // the reference's expression, as the compiler evaluates it: float
  // subtractions inside, everything else in double
  return (float)(p1 + 0.5 * x * ((float)(p2 - p0) + x * (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3 +
                                                         x * (3.0 * (float)(p1 - p2) + p3 - p0))));
}

static float grow_double(float v0, float v1, float v2, float v3, double t, double t2, double t3) {
  // the flow pyramid's growth, as CImg evaluates it in double
  const double val0 = v0, val1 = v1, val2 = v2, val3 = v3;
  const double val = val1 + 0.5f * (t * (-val0 + val2) + t2 * (2 * val0 - 5 * val1 + 4 * val2 - val3) +
                                    t3 * (-val0 + 3 * val1 - 3 * val2 + val3));
  return (float)val;
}

static uint64_t s_state;
static uint64_t rnd() {  // splitmix64
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unif() { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); }
static float bitsf(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static uint32_t fbits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

// A value of the kind the correction image holds, by mode.
static float sample(int mode, float base) {
  switch (mode) {
    case 0: return (float)((unif() * 2.0 - 1.0) * 10.0);                         // O(1)
    case 1: return (float)((unif() * 2.0 - 1.0) * pow(10.0, unif() * 12.0 - 8.0));  // wide magnitudes
    case 2: return base + (float)((unif() * 2.0 - 1.0) * fabs(base) * 1e-6);     // near-equal (cancellation)
    case 3: return (rnd() & 1) ? base : -base;                                    // ties, exact symmetry
    case 4: {                                                                      // random finite bit patterns
      uint32_t u;
      do u = (uint32_t)rnd(); while (((u >> 23) & 0xff) == 0xff);
      return bitsf(u);
    }
    default: return (float)(rnd() % 7) - 3.0f;                                    // small integers
  }
}

int main(int argc, char **argv) {
  const long long cases = argc > 1 ? atoll(argv[1]) : 20000000;
  s_state = argc > 2 ? strtoull(argv[2], 0, 10) : 12345;
  long long claimed = 0, bad = 0, u_claimed = 0, u_bad = 0, g_claimed = 0, g_bad = 0;
  const double alpha = 0.1;  // the reference's default -a
  const float ah = (float)alpha, al = (float)(alpha - (double)ah);
  for (long long c = 0; c < cases; ++c) {
    const int mode = (int)(rnd() % 6);
    const float base = (float)((unif() * 2.0 - 1.0) * 5.0);
    const float p0 = sample(mode, base), p1 = sample(mode, base), p2 = sample(mode, base), p3 = sample(mode, base);
    float x = (float)((double)(rnd() & ((1u << 22) - 1)) / 4194304.0);  // k 2^-22 in [0, 1)
    if ((rnd() & 15) == 0) x = 0.0f;
    if ((rnd() & 15) == 1) x = 0.5f;
    float got;
    if (wap::bpc::cubic_cert(p0, p1, p2, p3, x, &got)) {
      ++claimed;
      const float want = cubic_double(p0, p1, p2, p3, x);
      if (fbits(got) != fbits(want)) {
        if (bad < 10)
          printf("cubic mismatch: p=(%a %a %a %a) x=%a got %a want %a\n", p0, p1, p2, p3, x, got, want);
        ++bad;
      }
    }
    {
      double t = unif();  // an accumulated offset's fraction, any double in [0, 1)
      if ((rnd() & 15) == 0) t = 0.0;
      if ((rnd() & 15) == 1) t = 0.5;
      const double t2 = t * t, t3 = t2 * t;
      float tp[6];
      const double w[3] = {t, t2, t3};
      for (int q = 0; q < 3; ++q) {
        tp[2 * q] = (float)w[q];
        tp[2 * q + 1] = (float)(w[q] - (double)tp[2 * q]);
      }
      if (wap::bpc::grow_cert(p0, p1, p2, p3, tp, &got)) {
        ++g_claimed;
        const float want = grow_double(p0, p1, p2, p3, t, t2, t3);
        if (fbits(got) != fbits(want)) {
          if (g_bad < 10)
            printf("grow mismatch: v=(%a %a %a %a) t=%a got %a want %a\n", p0, p1, p2, p3, t, got, want);
          ++g_bad;
        }
      }
    }
    const float v = fabsf(sample(mode == 4 ? 0 : mode, base));
    const float g = sample(mode, base);
    if (wap::bpc::update_cert(v, g, ah, al, &got)) {
      ++u_claimed;
      const float want = (float)((double)v + alpha * (double)g);
      if (fbits(got) != fbits(want)) {
        if (u_bad < 10) printf("update mismatch: v=%a g=%a got %a want %a\n", v, g, got, want);
        ++u_bad;
      }
    }
  }
  printf("cases=%lld cubic-claimed=%lld cubic-mismatch=%lld update-claimed=%lld update-mismatch=%lld "
         "grow-claimed=%lld grow-mismatch=%lld\n",
         cases, claimed, bad, u_claimed, u_bad, g_claimed, g_bad);
  return (bad || u_bad || g_bad) ? 1 : 0;
}
