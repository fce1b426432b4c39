// Semi-Lagrangian warp of a volume by a flow field: advection::advect
// (advection.h:10-146) with CImg's _cubic_atXYZ (CImg.h:13429-13524).
//
// Per voxel: a BFECC-style back-trace p2 = p - dt v(p), p0 = p2 + dt v(p2),
// q = p2 + (p - p0)/2, then a Catmull-Rom tricubic sample at q limited to the
// min/max of its 8 trilinear neighbours.  Three clamped-tricubic samples per
// voxel (two of the 3-channel velocity, one of the source), 72 taps each, all
// FP32 without contraction so the result matches the reference bit for bit.
// The world position of each cell centre involves a double division in the
// reference (cell_grid_to_world); it is tabulated per axis on the host.
#include <algorithm>
#include <vector>

#include "f32x2.h"
#include "wap_internal.h"

namespace wap {
namespace {

struct Grid3 {
  int n[3];
  float a0[3], a1[3];  // aabb lower/upper per axis
};

// CImg's cubic kernel, float (CImg.h:13437-13519).  FAST (the precision
// form): the same polynomial in Horner form with fused multiply-adds, which
// rounds differently.
template <bool FAST>
__device__ __forceinline__ float cubf(float p, float c, float n, float a, float t) {
  if (FAST) {
    const float A = n - p;
    const float B = __fmaf_rn(2.0f, p, __fmaf_rn(-5.0f, c, __fmaf_rn(4.0f, n, -a)));
    const float C = __fmaf_rn(3.0f, c - n, a - p);
    return __fmaf_rn(0.5f * t, __fmaf_rn(__fmaf_rn(C, t, B), t, A), c);
  }
  return c + 0.5f * (t * (-p + n) + t * t * (2 * p - 5 * c + 4 * n - a) + t * t * t * (-p + 3 * c - 3 * n + a));
}

// cubf on two independent lanes at once (packed FP32, the same operations
// and order per lane, hence the same bits): two rows of one channel, or one
// row of two channels.  tt and ttt are t*t and (t*t)*t, as cubf forms them;
// nz is -0 in both lanes, from a kernel argument (products are fused
// multiply-adds onto it: f32x2.h).
template <bool FAST>
__device__ __forceinline__ f2 cubf2(f2 p, f2 c, f2 n, f2 a, f2 t, f2 tt, f2 ttt, f2 nz) {
  auto K = [](float k) { return f2_splat(k); };
  if (FAST) {
    const f2 A = f2_sub(n, p);
    const f2 B = f2_fma(K(2.0f), p, f2_fma(K(-5.0f), c, f2_fma(K(4.0f), n, f2_mul(K(-1.0f), a, nz))));
    const f2 C = f2_fma(K(3.0f), f2_sub(c, n), f2_sub(a, p));
    return f2_fma(f2_mul(K(0.5f), t, nz), f2_fma(f2_fma(C, t, B), t, A), c);
  }
  // -p + n is n - p, and -p + 3c is 3c - p, exactly (IEEE addition commutes)
  const f2 x1 = f2_mul(t, f2_sub(n, p), nz);
  const f2 b = f2_sub(f2_add(f2_sub(f2_mul(K(2.0f), p, nz), f2_mul(K(5.0f), c, nz)), f2_mul(K(4.0f), n, nz)), a);
  const f2 d = f2_add(f2_sub(f2_sub(f2_mul(K(3.0f), c, nz), p), f2_mul(K(3.0f), n, nz)), a);
  const f2 s = f2_add(f2_add(x1, f2_mul(tt, b, nz)), f2_mul(ttt, d, nz));
  return f2_add(c, f2_mul(K(0.5f), s, nz));
}

struct SamplePoint {
  int ix, iy, iz;    // trilinear cell for the limiter (advection.h:63)
  int xs[4], ys[4], zs[4];
  float dx, dy, dz;
};

// world_to_cell_grid + clamp to [1, n-2] (advection.h:32-36, 54-63) and
// CImg's tap indices (CImg.h:13431-13439).
__device__ __forceinline__ SamplePoint locate(const Grid3 &G, float px, float py, float pz) {
  const float p[3] = {px, py, pz};
  float g[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    // (float)((double)t - 0.5) is the float subtraction t - 0.5f.
    const float t = (float)G.n[a] * (p[a] - G.a0[a]) / (G.a1[a] - G.a0[a]);
    g[a] = t - 0.5f;
    g[a] = std_max(1.0f, std_min((float)(G.n[a] - 2), g[a]));
  }
  SamplePoint s;
  s.ix = (int)g[0];
  s.iy = (int)g[1];
  s.iz = (int)g[2];
  int *idx[3] = {s.xs, s.ys, s.zs};
  float *fr[3] = {&s.dx, &s.dy, &s.dz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float hi = (float)(G.n[a] - 1);
    const float nf = g[a] < 0.0f ? 0.0f : (g[a] > hi ? hi : g[a]);
    const int x = (int)nf;
    const float d = nf - (float)x;
    *fr[a] = d;
    idx[a][0] = x - 1 < 0 ? 0 : x - 1;
    idx[a][1] = x;
    idx[a][2] = d > 0.0f ? x + 1 : x;
    idx[a][3] = x + 2 >= G.n[a] ? G.n[a] - 1 : x + 2;
  }
  return s;
}

// sample_image (advection.h:49-88) of one channel at a located point.
template <bool FAST>
__device__ __forceinline__ float sample(const float *__restrict__ img, const Grid3 &G, const SamplePoint &s, f2 nz) {
  const int nx = G.n[0], nxy = G.n[0] * G.n[1];
  auto I = [&](int x, int y, int z) { return __ldg(img + (x + nx * y + nxy * z)); };
  float mn = I(s.ix, s.iy, s.iz), mx = mn;
  const int o[7][3] = {{1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const float v = I(s.ix + o[q][0], s.iy + o[q][1], s.iz + o[q][2]);
    mn = std_min(mn, v);
    mx = std_max(mx, v);
  }
  // One z plane of 16 taps per loop trip (not unrolled): the loads in flight
  // stay at 16 per thread, which keeps the register count low enough for
  // several blocks per SM; the arithmetic and its order are unchanged.
  // The x cubics of rows (0, 1) and (2, 3) run in pairs.
  const f2 t = f2_splat(s.dx), tt = f2_mul(t, t, nz), ttt = f2_mul(tt, t, nz);
  float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f, p3 = 0.0f;
#pragma unroll 1
  for (int kz = 0; kz < 4; ++kz) {
    const int z = kz == 0 ? s.zs[0] : kz == 1 ? s.zs[1] : kz == 2 ? s.zs[2] : s.zs[3];
    f2 rows[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int ya = s.ys[2 * h], yb = s.ys[2 * h + 1];
      auto tap = [&](int q) { return f2_pack(I(s.xs[q], ya, z), I(s.xs[q], yb, z)); };
      rows[h] = cubf2<FAST>(tap(0), tap(1), tap(2), tap(3), t, tt, ttt, nz);
    }
    const float pl = cubf<FAST>(f2_lo(rows[0]), f2_hi(rows[0]), f2_lo(rows[1]), f2_hi(rows[1]), s.dy);
    p0 = kz == 0 ? pl : p0;
    p1 = kz == 1 ? pl : p1;
    p2 = kz == 2 ? pl : p2;
    p3 = kz == 3 ? pl : p3;
  }
  const float c = cubf<FAST>(p0, p1, p2, p3, s.dz);
  return std_max(mn, std_min(mx, c));
}

// The three velocity channels at one located point: the same taps, limiter
// and arithmetic per channel as three sample() calls, in one pass over the
// taps so the index arithmetic is shared and the channels' loads interleave.
template <bool FAST>
__device__ __forceinline__ void sample3(const float *__restrict__ vel, size_t nv, const Grid3 &G,
                                        const SamplePoint &s, float out[3], f2 nz) {
  const int nx = G.n[0], nxy = G.n[0] * G.n[1];
  auto at = [&](int x, int y, int z) { return x + nx * y + nxy * z; };
  float mn[3], mx[3];
  {
    const int i0 = at(s.ix, s.iy, s.iz);
#pragma unroll
    for (int c = 0; c < 3; ++c) mn[c] = mx[c] = __ldg(vel + c * nv + i0);
  }
  const int o[7][3] = {{1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const int i = at(s.ix + o[q][0], s.iy + o[q][1], s.iz + o[q][2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = __ldg(vel + c * nv + i);
      mn[c] = std_min(mn[c], v);
      mx[c] = std_max(mx[c], v);
    }
  }
  // Channels 0 and 1 run in pairs through all three cubic stages, channel 2
  // in scalars.
  const f2 tx = f2_splat(s.dx), ttx = f2_mul(tx, tx, nz), tttx = f2_mul(ttx, tx, nz);
  const f2 ty = f2_splat(s.dy), tty = f2_mul(ty, ty, nz), ttty = f2_mul(tty, ty, nz);
  const float *ch0 = vel, *ch1 = vel + nv, *ch2 = vel + 2 * nv;
  f2 p01[4];
  float p2[4];
#pragma unroll 1
  for (int kz = 0; kz < 4; ++kz) {
    const int z = kz == 0 ? s.zs[0] : kz == 1 ? s.zs[1] : kz == 2 ? s.zs[2] : s.zs[3];
    f2 rows01[4];
    float rows2[4];
#pragma unroll
    for (int ky = 0; ky < 4; ++ky) {
      const int r = at(0, s.ys[ky], z);
      const int i0 = r + s.xs[0], i1 = r + s.xs[1], i2 = r + s.xs[2], i3 = r + s.xs[3];
      auto tap = [&](int i) { return f2_pack(__ldg(ch0 + i), __ldg(ch1 + i)); };
      rows01[ky] = cubf2<FAST>(tap(i0), tap(i1), tap(i2), tap(i3), tx, ttx, tttx, nz);
      rows2[ky] = cubf<FAST>(__ldg(ch2 + i0), __ldg(ch2 + i1), __ldg(ch2 + i2), __ldg(ch2 + i3), s.dx);
    }
    const f2 pl01 = cubf2<FAST>(rows01[0], rows01[1], rows01[2], rows01[3], ty, tty, ttty, nz);
    const float pl2 = cubf<FAST>(rows2[0], rows2[1], rows2[2], rows2[3], s.dy);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      p01[q] = kz == q ? pl01 : p01[q];
      p2[q] = kz == q ? pl2 : p2[q];
    }
  }
  const f2 tz = f2_splat(s.dz), ttz = f2_mul(tz, tz, nz), tttz = f2_mul(ttz, tz, nz);
  const f2 r01 = cubf2<FAST>(p01[0], p01[1], p01[2], p01[3], tz, ttz, tttz, nz);
  const float r[3] = {f2_lo(r01), f2_hi(r01), cubf<FAST>(p2[0], p2[1], p2[2], p2[3], s.dz)};
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = std_max(mn[c], std_min(mx[c], r[c]));
}

// 1 in bad[j] when job j's velocity field has a component that is NaN or
// has |v| >= 2^124 (the advect kernel's centre shortcut needs neither).
__global__ void __launch_bounds__(256) vel_range_kernel(const AdvectJob *__restrict__ jobs, size_t n3, int *bad) {
  const float *__restrict__ v = jobs[blockIdx.y].vel;
  int b = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n3; i += (size_t)gridDim.x * blockDim.x)
    b |= (__float_as_uint(__ldg(v + i)) & 0x7fffffffu) >= 0x7d800000u;
  if (__syncthreads_or(b) && threadIdx.x == 0) bad[blockIdx.y] = 1;
}

// The velocity at a sample point that sits exactly on a cell centre (every
// interpolation weight zero): there each of CImg's cubics c + 0.5 (t (..) +
// t^2 (..) + t^3 (..)) with t = 0, and the Horner form of the precision
// form, is its centre tap c, as long as no bracketed term is NaN or
// overflows (the taps are below 2^124 in magnitude, so each term stays below
// 12 * 2^124 < 2^128), up to the sign of a zero result; and the limiter
// keeps c, which is one of its 8 cells.  The trace uses the velocity only as
// p + dt v with p a positive cell-centre coordinate, so a zero's sign cannot
// change the output: the centre tap gives the reference's bits.
template <bool FAST>
__global__ void __launch_bounds__(128, 6) advect_kernel(Grid3 G, const float *__restrict__ wx,
                                                     const float *__restrict__ wy, const float *__restrict__ wz,
                                                     const AdvectJob *__restrict__ jobs, int nc,
                                                     const int *__restrict__ bad, float negzero) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z % G.n[2];
  const int jb = blockIdx.z / G.n[2];
  const AdvectJob job = jobs[jb];
  if (i >= G.n[0] || j >= G.n[1]) return;
  const bool centre_ok = bad && !bad[jb];
  const f2 nz = f2_splat(negzero);
  const float *__restrict__ vel = job.vel;
  const float *__restrict__ src = job.src;
  float *__restrict__ out = job.out;
  const float tdt = -job.dt;
  const size_t nv = (size_t)G.n[0] * G.n[1] * G.n[2];
  const float p[3] = {__ldg(wx + i), __ldg(wy + j), __ldg(wz + k)};
  // trace (advection.h:101-115) with dt_trace = -dt.
  SamplePoint s = locate(G, p[0], p[1], p[2]);
  float v[3];
  if (centre_ok && s.dx == 0.0f && s.dy == 0.0f && s.dz == 0.0f) {
    const size_t c = s.xs[1] + (size_t)G.n[0] * (s.ys[1] + (size_t)G.n[1] * s.zs[1]);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) v[ch] = __ldg(vel + ch * nv + c);
  } else {
    sample3<FAST>(vel, nv, G, s, v, nz);
  }
  const float p2[3] = {p[0] + tdt * v[0], p[1] + tdt * v[1], p[2] + tdt * v[2]};
  s = locate(G, p2[0], p2[1], p2[2]);
  sample3<FAST>(vel, nv, G, s, v, nz);
  const float p0[3] = {p2[0] - tdt * v[0], p2[1] - tdt * v[1], p2[2] - tdt * v[2]};
  const float q[3] = {p2[0] + (p[0] - p0[0]) * 0.5f, p2[1] + (p[1] - p0[1]) * 0.5f, p2[2] + (p[2] - p0[2]) * 0.5f};
  s = locate(G, q[0], q[1], q[2]);
  const size_t o = i + (size_t)G.n[0] * (j + (size_t)G.n[1] * k);
  for (int c = 0; c < nc; ++c) out[c * nv + o] = sample<FAST>(src + c * nv, G, s, nz);
}

// vol += alpha * adv (double, CImg operator* / operator+=), cut(0, G_Max),
// then max(vol * imROI, 0) with imROI == 1 (WaP_Tomo.cpp:1378-1412).
// FLOOR = false: the cut alone (AdaptiveWarp, WaP_Tomo.cpp:1160-1161, floors once at its end).
template <bool FLOOR>
__global__ void wap_accumulate_kernel(size_t n, float *__restrict__ vol, const float *__restrict__ adv, double alpha,
                                      float gmax) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = (float)((double)vol[i] + (double)adv[i] * alpha);
  x = (x < 0.0f) ? 0.0f : ((x > gmax) ? gmax : x);
  vol[i] = FLOOR ? mac_max(x * 1.0f, 0.0f) : x;
}

__global__ void wap_accumulate_batch_kernel(const AccJob *__restrict__ jobs, size_t n, double alpha, float gmax) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const AccJob jb = jobs[blockIdx.y];
  float x = (float)((double)jb.vol[i] + (double)jb.adv[i] * alpha);
  x = (x < 0.0f) ? 0.0f : ((x > gmax) ? gmax : x);
  jb.vol[i] = mac_max(x * 1.0f, 0.0f);
}

__global__ void roi_floor_kernel(size_t n, float *__restrict__ vol) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  vol[i] = mac_max(vol[i] * 1.0f, 0.0f);
}

// Self-check of the packed cubic: per index, CImg's cubic on two lanes of
// pseudo-random inputs (any float bits, small dyadic values, tiny and
// subnormal values, signed zeros; t mostly in [0, 1) as the warp's
// fractions are) in scalars and in one packed pair, both arithmetics; counts
// the results whose bits differ (NaN against NaN counts as equal).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {  // splitmix64 finaliser
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float check_input(unsigned long long h, bool is_t) {
  const unsigned b = (unsigned)h, kind = (unsigned)(h >> 32) & 7u, sign = (unsigned)(h >> 35) & 1u;
  if (is_t && kind < 4) return (float)(b >> 8) * 0x1p-24f;  // [0, 1); else any of the kinds below
  switch (kind) {
    case 0: return __uint_as_float(b);                                      // any bits
    case 1: return __uint_as_float((b & 0x007fffffu) | (sign << 31));      // subnormal or zero
    case 2: return sign ? -0.0f : 0.0f;
    case 3: return (float)(int)(b & 0xffffu) * 0x1p-12f * (sign ? -1.0f : 1.0f);  // dyadic
    case 4: return __uint_as_float((b & 0x807fffffu) | (0x00800000u + (b & 0x07000000u)));  // tiny normal
    default: return __uint_as_float((b & 0x807fffffu) | (((120u + ((b >> 23) & 15u)) & 0xffu) << 23));  // ~1
  }
}
__device__ __forceinline__ bool same_bits(float a, float b) {
  return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}
__global__ void cubic_pair_check_kernel(unsigned long long n, unsigned long long seed, float negzero,
                                        unsigned long long *bad) {
  const f2 nz = f2_splat(negzero);
  unsigned long long cnt = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    float v[2][5];
#pragma unroll
    for (int l = 0; l < 2; ++l)
#pragma unroll
      for (int q = 0; q < 5; ++q) v[l][q] = check_input(mix64(seed + 10 * i + 5 * l + q), q == 4);
    const f2 p = f2_pack(v[0][0], v[1][0]), c = f2_pack(v[0][1], v[1][1]), m = f2_pack(v[0][2], v[1][2]),
             a = f2_pack(v[0][3], v[1][3]);
    // the pair's t differs per lane here (in the warp both lanes share one t)
    const f2 t = f2_pack(v[0][4], v[1][4]), tt = f2_mul(t, t, nz), ttt = f2_mul(tt, t, nz);
    const f2 r = cubf2<false>(p, c, m, a, t, tt, ttt, nz), rf = cubf2<true>(p, c, m, a, t, tt, ttt, nz);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const float e = cubf<false>(v[l][0], v[l][1], v[l][2], v[l][3], v[l][4]);
      const float ef = cubf<true>(v[l][0], v[l][1], v[l][2], v[l][3], v[l][4]);
      cnt += !same_bits(l ? f2_hi(r) : f2_lo(r), e);
      cnt += !same_bits(l ? f2_hi(rf) : f2_lo(rf), ef);
    }
  }
  if (cnt) atomicAdd(bad, cnt);
}

}  // namespace

cudaError_t launch_cubic_pair_check(unsigned long long n, unsigned long long seed, unsigned long long *d_bad,
                                    cudaStream_t st) {
  cubic_pair_check_kernel<<<152 * 8, 256, 0, st>>>(n, seed, -0.0f, d_bad);
  return cudaGetLastError();
}

void world_table(const int dims[3], const float aabb[6], float *h) {
  int off = 0;
  for (int a = 0; a < 3; ++a) {
    for (int i = 0; i < dims[a]; ++i) {
      const float gf = (float)i;
      h[off + i] = (float)(aabb[2 * a] + (gf + 0.5) * (aabb[2 * a + 1] - aabb[2 * a]) / (float)dims[a]);
    }
    off += dims[a];
  }
}

cudaError_t launch_advect(const int dims[3], const float aabb[6], const float *d_world, const AdvectJob *d_jobs,
                          int njobs, int nc, cudaStream_t st, bool fast, int *d_flags) {
  if (njobs <= 0) return cudaSuccess;
  if (d_flags) {  // the range check of each job's velocity (the centre shortcut's condition)
    cudaError_t e = cudaMemsetAsync(d_flags, 0, sizeof(int) * njobs, st);
    if (e != cudaSuccess) return e;
    const size_t n3 = 3 * (size_t)dims[0] * dims[1] * dims[2];
    const unsigned gx = (unsigned)std::min<size_t>((n3 + 255) / 256, 1216);
    for (int j = 0; j < njobs; j += 65535) {
      vel_range_kernel<<<dim3(gx, (unsigned)std::min(65535, njobs - j)), 256, 0, st>>>(d_jobs + j, n3, d_flags + j);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  Grid3 G;
  for (int a = 0; a < 3; ++a) {
    G.n[a] = dims[a];
    G.a0[a] = aabb[2 * a];
    G.a1[a] = aabb[2 * a + 1];
  }
  const dim3 block(32, 4, 1);
  // jobs x z planes go in gridDim.z; more than 65535 are split into launches
  // of whole jobs
  const int per = std::max(1, 65535 / dims[2]);
  for (int j = 0; j < njobs; j += per) {
    const int n = std::min(per, njobs - j);
    const dim3 grid((dims[0] + 31) / 32, (dims[1] + 3) / 4, dims[2] * n);
    const int *bad = d_flags ? d_flags + j : nullptr;
    if (fast)
      advect_kernel<true><<<grid, block, 0, st>>>(G, d_world, d_world + dims[0], d_world + dims[0] + dims[1], d_jobs + j,
                                                  nc, bad, -0.0f);
    else
      advect_kernel<false><<<grid, block, 0, st>>>(G, d_world, d_world + dims[0], d_world + dims[0] + dims[1],
                                                   d_jobs + j, nc, bad, -0.0f);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_wap_accumulate(size_t n, float *vol, const float *adv, double alpha, float gmax, cudaStream_t st,
                                  bool floor) {
  if (floor) wap_accumulate_kernel<true><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, vol, adv, alpha, gmax);
  else wap_accumulate_kernel<false><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, vol, adv, alpha, gmax);
  return cudaGetLastError();
}

cudaError_t launch_wap_accumulate_batch(const AccJob *d_jobs, int njobs, size_t n, double alpha, float gmax,
                                        cudaStream_t st) {
  if (njobs <= 0) return cudaSuccess;
  const dim3 g((unsigned)((n + 255) / 256), njobs);
  wap_accumulate_batch_kernel<<<g, 256, 0, st>>>(d_jobs, n, alpha, gmax);
  return cudaGetLastError();
}

cudaError_t launch_roi_floor(size_t n, float *vol, cudaStream_t st) {
  roi_floor_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, vol);
  return cudaGetLastError();
}

}  // namespace wap
