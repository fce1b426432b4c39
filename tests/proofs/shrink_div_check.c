/* Exhaustive host check of the primal-dual kernels' division-free shrink
 * (pd::shrink_fast and pd::shrink_tiny in
 * warp-and-project-tomography_gb300/csrc/flow.cu, restated operation for
 * operation with C99 fmaf, no contraction, subnormals on): over all 2^32 float
 * inputs a, the fast path where its guard accepts a and the scaled path for
 * 0 < |a| < 1e-30 must give the bits of the IEEE quotient a / den.  The GPU
 * repeats the same proof on the device before it uses the fast path; this
 * host run pins the algorithm for a range of lambdas without a GPU.  With
 * the argument "sigma1" the divisor is sigma1 itself, which the residual
 * iterations divide nine dual terms by.
 * Prints the mismatch counts; exit status 1 if any. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <stdlib.h>
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
/* noinline: each candidate is evaluated as the scalar sequence written here. */
__attribute__((noinline)) static float shrink_fast(float a, float den, float rinv, int *bad) {
  const float q0 = a * rinv;
  const float en = fmaf(q0, den, -a);
  const float q = fmaf(-en, rinv, q0);
  *bad |= (a != 0.0f && fabsf(a) < 1.0e-30f) || !(fabsf(q0) < 3.0e38f);
  return q;
}
__attribute__((noinline)) static float shrink_tiny(float a, float den, float rinv) {
  const float a2 = a * 0x1p64f;
  const float q0 = a2 * rinv;
  const float q2 = fmaf(fmaf(-q0, den, a2), rinv, q0);
  const float e = fmaf(-q2, den, a2);
  float t = q2 * 0x1p-64f;
  const float d = q2 - t * 0x1p64f;
  if (fabsf(d) == 0x1p-86f && e != 0.0f && ((d > 0.0f) == (e > 0.0f))) t += e > 0.0f ? 0x1p-149f : -0x1p-149f;
  return t;
}
int main(int argc, char **argv) {
  const int by_sigma1 = argc > 1 && strcmp(argv[1], "sigma1") == 0;
  const float lambda = argc > 1 && !by_sigma1 ? strtof(argv[1], 0) : 0.05f;
  const float sigma1 = 1.0f / 3.0f;
  const float den = by_sigma1 ? sigma1 : lambda + 2 * sigma1, rinv = 1.0f / den;
  unsigned long long bad_fast = 0, bad_tiny = 0, n_tiny = 0, n_ieee = 0;
  #pragma omp parallel for reduction(+:bad_fast,bad_tiny,n_tiny,n_ieee) schedule(static)
  for (long long i = 0; i < (1LL << 32); ++i) {
    const float a = u2f((uint32_t)i);
    const float ref = a / den;
    int bad = 0;
    float r = shrink_fast(a, den, rinv, &bad);
    if (!bad) {
      if (!(f2u(r) == f2u(ref) || (r != r && ref != ref))) {
        ++bad_fast;
        fprintf(stderr, "fast mismatch: a=%08x (%.9g) fast=%08x ieee=%08x\n", (unsigned)i, a, f2u(r), f2u(ref));
      }
      continue;
    }
    if (a != 0.0f && fabsf(a) < 1.0e-30f) {
      ++n_tiny;
      r = shrink_tiny(a, den, rinv);
      if (!(f2u(r) == f2u(ref))) {
        ++bad_tiny;
        fprintf(stderr, "tiny mismatch: a=%08x (%.9g) fast=%08x ieee=%08x\n", (unsigned)i, a, f2u(r), f2u(ref));
      }
    } else ++n_ieee;
  }
  printf("den=%.9g fast-mismatch=%llu tiny=%llu tiny-mismatch=%llu ieee=%llu\n", den, bad_fast, n_tiny, bad_tiny, n_ieee);
  return (bad_fast || bad_tiny) ? 1 : 0;
}
