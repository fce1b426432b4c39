// Pairs of FP32 values operated on by the packed FP32 instructions of sm_100
// and later (add/sub/fma .rn .f32x2).  Each lane of a packed instruction is
// rounded exactly as the scalar instruction, so an expression evaluated
// lane-wise in pairs gives the bits of the same expression in scalars, with
// one caveat: ptxas contracts a packed multiply and a following packed add or
// subtract into a packed fused multiply-add, even under .rn and --fmad=false
// (measured: 3c - p came out as fma(3, c, -p) in a fifth of random cases).
// So a product is formed here only as fma(a, b, z) with z = -0 passed in at
// run time from a kernel argument: a*b + (-0) rounds to the rounding of a*b
// for every a and b (a product of +0 stays +0, of -0 stays -0), and ptxas,
// not knowing z, can neither turn it back into a plain multiply nor fuse it
// with the add that follows.  A packed instruction takes one issue slot for
// two results (the FMA pipe does the same work as for two scalars), which is
// what the issue-bound kernels gain.
#pragma once

namespace wap {

struct f2 {
  unsigned long long r;
};

__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
  f2 v;
  asm("mov.b64 %0, {%1, %2};" : "=l"(v.r) : "f"(lo), "f"(hi));
  return v;
}
__device__ __forceinline__ f2 f2_splat(float x) { return f2_pack(x, x); }
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v.r));
}
__device__ __forceinline__ float f2_lo(f2 v) {
  float lo, hi;
  f2_unpack(v, lo, hi);
  return lo;
}
__device__ __forceinline__ float f2_hi(f2 v) {
  float lo, hi;
  f2_unpack(v, lo, hi);
  return hi;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
  return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
  return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.r) : "l"(a.r), "l"(b.r), "l"(c.r));
  return d;
}

// a * b rounded once; nz must be -0 in both lanes, from a kernel argument.
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b, f2 nz) { return f2_fma(a, b, nz); }

}  // namespace wap
