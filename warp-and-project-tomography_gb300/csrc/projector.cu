// Cone-beam projector kernels: ray-driven forward projection (with the fused
// PSART correction epilogue), the voxel-driven bicubic backprojection, and
// the ray-driven matched backprojection (splat).
//
// Forward projection restates GenerateImage_MT / ProduceRay / CastingRay /
// T_VolumeAccess::GetScalarValue (TypicalRayProducer.core.h:32-225,
// RayCaster.core.h:42-188, SingleScalarVolume.core.h:66-202) one thread per
// detector pixel: the reference's march accumulates t and pos in float and
// re-derives t at every block boundary, so the sample positions (and with them
// the sample counts) are a sequential recurrence that must be replayed, not
// reformulated.  Each warp owns an 8x4 pixel patch so the warp's 32 rays stay
// within a few voxels of each other and the trilinear gathers hit L1.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include <cuda_fp16.h>

#include "bp_cubic.h"
#include "wap_internal.h"

namespace wap {
namespace {

struct VolView {
  const float *__restrict__ d;
  int nx, ny, nz;
  __device__ __forceinline__ float at(int x, int y, int z) const {
    // T_VolumeAccess::GetScalarValue(int,int,int): clamp each index to [0, n-1].
    x = mac_maxi(mac_mini(x, nx - 1), 0);
    y = mac_maxi(mac_mini(y, ny - 1), 0);
    z = mac_maxi(mac_mini(z, nz - 1), 0);
    return __ldg(d + (x + nx * (y + ny * z)));
  }
};

// The same volume as 4x4x4 bricks of 64 floats (bricks x-fastest, each brick
// z-major inside), so the 32 rays of a warp, which sample a small patch of a
// plane across the ray direction, gather from a few 256-byte bricks instead
// of many x rows.  Same clamping, same values: only the address changes.
// T = __half: the precision form's FP16 copy (the taps widen to FP32).
template <class T>
struct BrickViewT {
  const T *__restrict__ d;
  int nx, ny, nz, nbx, nby;
  // The 8 trilinear taps of cell (i, j, k), 0 <= i < nx etc., in the
  // sampler's order, each index +1 clamped to n-1 as VolView::at does: one
  // brick address (cell (x, y, z) sits at brick ((z/4) nby + y/4) nbx + x/4,
  // offset 16 (z%4) + 4 (y%4) + x%4) and a step per axis (within the brick,
  // into the next brick, or 0 at the last cell).
  __device__ __forceinline__ void taps8(int i, int j, int k, float t[8]) const {
    const size_t b = ((size_t)(k >> 2) * nby + (j >> 2)) * nbx + (i >> 2);
    const T *p = d + (b << 6) + ((k & 3) << 4) + ((j & 3) << 2) + (i & 3);
    const int sx = i + 1 > nx - 1 ? 0 : ((i & 3) == 3 ? 61 : 1);
    const int sy = j + 1 > ny - 1 ? 0 : ((j & 3) == 3 ? nbx * 64 - 12 : 4);
    const int sz = k + 1 > nz - 1 ? 0 : ((k & 3) == 3 ? nbx * nby * 64 - 48 : 16);
    t[0] = ld(p);
    t[1] = ld(p + sx);
    t[2] = ld(p + sy);
    t[3] = ld(p + sx + sy);
    t[4] = ld(p + sz);
    t[5] = ld(p + sx + sz);
    t[6] = ld(p + sy + sz);
    t[7] = ld(p + sx + sy + sz);
  }
  static __device__ __forceinline__ float ld(const float *p) { return __ldg(p); }
  static __device__ __forceinline__ float ld(const __half *p) { return __half2float(__ldg(p)); }
};
using BrickView = BrickViewT<float>;
using BrickViewH = BrickViewT<__half>;
template <class V>
struct is_brick : std::false_type {};
template <class T>
struct is_brick<BrickViewT<T>> : std::true_type {};

// Trilinear sample with the reference's clamp-then-truncate (SingleScalarVolume.core.h:99-202).
template <class View>
struct TrilinearSampler {
  View v;
  float sumw;
  __device__ __forceinline__ float operator()(float p0, float p1, float p2) {
    p0 = mac_max(mac_min(p0, (float)(v.nx - 1)), 0.0f);
    p1 = mac_max(mac_min(p1, (float)(v.ny - 1)), 0.0f);
    p2 = mac_max(mac_min(p2, (float)(v.nz - 1)), 0.0f);
    const int i = (int)p0, j = (int)p1, k = (int)p2;
    float f2 = p0 - (float)i;
    float f1 = 1.0f - f2;
    sumw += 1.0f;
    float tp[8];
    if constexpr (is_brick<View>::value) {
      v.taps8(i, j, k, tp);
    } else {
      tp[0] = v.at(i, j, k);
      tp[1] = v.at(i + 1, j, k);
      tp[2] = v.at(i, j + 1, k);
      tp[3] = v.at(i + 1, j + 1, k);
      tp[4] = v.at(i, j, k + 1);
      tp[5] = v.at(i + 1, j, k + 1);
      tp[6] = v.at(i, j + 1, k + 1);
      tp[7] = v.at(i + 1, j + 1, k + 1);
    }
    float a = tp[0] * f1 + tp[1] * f2;
    float b = tp[2] * f1 + tp[3] * f2;
    float c = tp[4] * f1 + tp[5] * f2;
    float d = tp[6] * f1 + tp[7] * f2;
    f2 = p1 - (float)j;
    f1 = 1.0f - f2;
    a = a * f1 + b * f2;
    c = c * f1 + d * f2;
    f2 = p2 - (float)k;
    f1 = 1.0f - f2;
    return a * f1 + c * f2;
  }
};

// Back-projection mode of the same sampler (SingleScalarVolume.core.h:85-96,
// 149-199): splat corr*w_k and w_k onto the 8 taps.  Taps past the last voxel
// carry weight 0 (the position is clamped to n-1) and are dropped.
struct SplatSampler {
  int nx, ny, nz;
  float corr;
  float *__restrict__ contrib;
  float *__restrict__ weight;
  float sumw;
  __device__ __forceinline__ float operator()(float p0, float p1, float p2) {
    p0 = mac_max(mac_min(p0, (float)(nx - 1)), 0.0f);
    p1 = mac_max(mac_min(p1, (float)(ny - 1)), 0.0f);
    p2 = mac_max(mac_min(p2, (float)(nz - 1)), 0.0f);
    const int i = (int)p0, j = (int)p1, k = (int)p2;
    const float t0 = p0 - (float)i, t1 = p1 - (float)j, t2 = p2 - (float)k;
    const float M0 = 1.0f - t0, M1 = 1.0f - t1, M2 = 1.0f - t2;
    const float w[8] = {M0 * M1 * M2, t0 * M1 * M2, M0 * t1 * M2, t0 * t1 * M2,
                        M0 * M1 * t2, t0 * M1 * t2, M0 * t1 * t2, t0 * t1 * t2};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int x = i + (c & 1), y = j + ((c >> 1) & 1), z = k + ((c >> 2) & 1);
      if (x >= nx || y >= ny || z >= nz) continue;
      const int id = x + nx * (y + ny * z);
      atomicAdd(contrib + id, corr * w[c]);
      atomicAdd(weight + id, w[c]);
    }
    return 0.0f;
  }
};

// ProduceRay (TypicalRayProducer.core.h:32-120).
__device__ __forceinline__ void produce_ray(const ProjGeom &g, int nx, int ny, int nz, float px, float py,
                                            float vz[4], float vu[4], float &tnear, float &tfar) {
  float mp[4];
  mat4_vec(g.p2m, px, py, 0.0f, 1.0f, mp);
  const float inv = 1.0f / mp[3];
#pragma unroll
  for (int a = 0; a < 4; ++a) mp[a] *= inv;
  float dir[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) dir[a] = mp[a] - g.eye[a];
  const float li = 1.0f / sqrtf(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
  dir[0] *= li;
  dir[1] *= li;
  dir[2] *= li;
  mat4_vec(g.m2v, g.eye[0], g.eye[1], g.eye[2], g.eye[3], vz);
  mat4_vec(g.m2v, dir[0], dir[1], dir[2], dir[3], vu);
  const float hi[3] = {(float)(nx - 1), (float)(ny - 1), (float)(nz - 1)};
  float tmn[3], tmx[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float t1 = (0.0f - vz[a]) / vu[a];
    const float t2 = (hi[a] - vz[a]) / vu[a];
    tmn[a] = mac_min(t1, t2);
    tmx[a] = mac_max(t1, t2);
  }
  tnear = mac_max(mac_max(tmn[0], tmn[1]), tmn[2]);
  tnear = mac_max(tnear, 0.0f);
  tfar = mac_min(mac_min(tmx[0], tmx[1]), tmx[2]);
}

// CastingRay with one block spanning the whole volume (RayCasterPrepare sets
// bsize = volume dims, RayCaster.core.h:191-207).
// KAHAN (the precision form's projector): the ray sum with Kahan's
// compensation, so the FP16 samples are summed without FP32 round-off growth.
template <class Sampler, bool KAHAN = false>
__device__ __forceinline__ float cast_ray(Sampler &smp, const int n[3], const float vz[4], const float vu[4],
                                          float tnear, float tfar, float sd) {
  float density = 0.0f, comp = 0.0f;
  auto add = [&](float v) {
    if (KAHAN) {
      const float y = v - comp;
      const float t = density + y;
      comp = (t - density) - y;
      density = t;
    } else {
      density += v;
    }
  };
  float t1 = tnear;
  const float pos1[3] = {vz[0] + vu[0] * t1, vz[1] + vu[1] * t1, vz[2] + vu[2] * t1};
  const float step[3] = {vu[0] * sd, vu[1] * sd, vu[2] * sd};
  add(smp(pos1[0], pos1[1], pos1[2]) * sd);
  float tMax[3], tDelta[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int bs = n[a];
    if (vu[a] == 0.0f) {
      tMax[a] = tfar;
    } else if (vu[a] < 0.0f) {
      const int blk = ((int)ceilf(pos1[a] - 0.5f) - 1) / bs;
      tMax[a] = ((float)(blk * bs) + 0.5f - vz[a]) / vu[a];
      tDelta[a] = (float)(-(1 * bs)) / vu[a];
    } else {
      const int blk = ((int)floorf(pos1[a] - 0.5f)) / bs;
      tMax[a] = ((float)((blk + 1) * bs) + 0.5f - vz[a]) / vu[a];
      tDelta[a] = (float)(1 * bs) / vu[a];
    }
  }
  while (t1 < tfar) {
    float tb = mac_min(mac_min(tMax[0], tMax[1]), tMax[2]);
    if (tb > tfar) tb = tfar;
    float t = ceilf((t1 - tnear) / sd) * sd + tnear;
    float p0 = vz[0] + vu[0] * t, p1 = vz[1] + vu[1] * t, p2 = vz[2] + vu[2] * t;
    while (t < tb) {
      add(smp(p0, p1, p2) * sd);
      t += sd;
      p0 += step[0];
      p1 += step[1];
      p2 += step[2];
    }
    if (tMax[0] < tMax[1]) {
      if (tMax[0] < tMax[2]) tMax[0] += tDelta[0];
      else tMax[2] += tDelta[2];
    } else {
      if (tMax[1] < tMax[2]) tMax[1] += tDelta[1];
      else tMax[2] += tDelta[2];
    }
    t1 = tb;
  }
  return density;
}

// Linear (x-fastest) volume -> the BrickView layout.  A 256-thread block
// moves a 32 x 4 x 4 tile: eight x-consecutive bricks, which are 2 KB in a
// row of the output, so the rows of the tile are read and the bricks written
// with whole-line accesses through shared memory.  Cells of partial bricks
// past the grid are written as 0 and never read (indices are clamped first).
template <class T>
__device__ __forceinline__ T to_store(float v);
template <>
__device__ __forceinline__ float to_store<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ __half to_store<__half>(float v) {
  return __float2half_rn(v);
}

template <class T>
__device__ __forceinline__ void brick_tile(const float *__restrict__ in, T *__restrict__ out, int nx, int ny,
                                           int nz, int x0, int y0, int z0, float (*t)[4][32]) {
  const int tid = threadIdx.x;
  for (int e = tid; e < 512; e += 256) {  // rows in: e = (z * 4 + y) * 32 + x
    const int x = e & 31, y = (e >> 5) & 3, z = e >> 7;
    const int gx = x0 + x, gy = y0 + y, gz = z0 + z;
    t[z][y][x] = (gx < nx && gy < ny && gz < nz) ? in[gx + (size_t)nx * (gy + (size_t)ny * gz)] : 0.0f;
  }
  __syncthreads();
  const int nbx = (nx + 3) >> 2, nby = (ny + 3) >> 2;
  const size_t b0 = ((size_t)(z0 >> 2) * nby + (y0 >> 2)) * nbx + (x0 >> 2);
  for (int o = tid; o < 512; o += 256) {  // bricks out: o = brick * 64 + (z * 4 + y) * 4 + x
    const int bx = o >> 6;
    if ((x0 >> 2) + bx >= nbx) continue;
    const int x = (o & 3) + 4 * bx, y = (o >> 2) & 3, z = (o >> 4) & 3;
    out[(b0 << 6) + o] = to_store<T>(t[z][y][x]);
  }
}

__global__ void __launch_bounds__(256) brick_kernel(const float *__restrict__ in, float *__restrict__ out, int nx,
                                                    int ny, int nz) {
  __shared__ float t[4][4][32];
  brick_tile(in, out, nx, ny, nz, blockIdx.x * 32, blockIdx.y * 4, blockIdx.z * 4, t);
}

// The volumes of n projection jobs (jobs[j].vol, linear) into consecutive
// brick-layout slots of bf floats; blockIdx.z runs over z tiles x jobs.
template <class T>
__global__ void __launch_bounds__(256) brick_jobs_kernel(const FpJob *__restrict__ jobs, T *__restrict__ out,
                                                         size_t bf, int nx, int ny, int nz, int ztiles) {
  __shared__ float t[4][4][32];
  const int j = blockIdx.z / ztiles;
  brick_tile(jobs[j].vol, out + j * bf, nx, ny, nz, blockIdx.x * 32, blockIdx.y * 4, (blockIdx.z % ztiles) * 4, t);
}

// 16x8 pixel tile per 128-thread block, each warp an 8x4 patch.
__device__ __forceinline__ void tile_pixel(int &i, int &j) {
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  i = blockIdx.x * 16 + (w & 1) * 8 + (lane & 7);
  j = blockIdx.y * 8 + (w >> 1) * 4 + (lane >> 3);
}

// One detector pixel (i, j) of a projection job: the ray, its march, the
// outputs and the fused correction.  Shared by the per-launch and the
// work-queue forms, so both compute the same bits.
template <class View>
__device__ __forceinline__ void fp_pixel(const ProjGeom *__restrict__ geom, const FpJob &job, int nx, int ny, int nz,
                                         int W, int H, float sd, double alpha, int i, int j) {
  const ProjGeom &g = geom[job.proj];
  const int n[3] = {nx, ny, nz};
  float vz[4], vu[4], tn, tf;
  produce_ray(g, nx, ny, nz, (float)i, (float)j, vz, vu, tn, tf);
  View view;
  if constexpr (std::is_same<View, BrickViewH>::value)
    view = BrickViewH{reinterpret_cast<const __half *>(job.vol), nx, ny, nz, (nx + 3) >> 2, (ny + 3) >> 2};
  else if constexpr (std::is_same<View, BrickView>::value)
    view = BrickView{job.vol, nx, ny, nz, (nx + 3) >> 2, (ny + 3) >> 2};
  else
    view = VolView{job.vol, nx, ny, nz};
  TrilinearSampler<View> smp{view, 0.0f};
  float value = 0.0f, len = 0.0f;
  if (tn < tf) {
    len = tf - tn;
    value = cast_ray<TrilinearSampler<View>, std::is_same<View, BrickViewH>::value>(smp, n, vz, vu, tn, tf, sd);
  }
  const int k = i + j * W;
  if (job.img) job.img[k] = value;
  if (job.len) job.len[k] = len;
  if (job.weight) job.weight[k] = smp.sumw;
  if (job.meas) {
    // PSART correction and dual (WaP_Tomo.cpp:1530-1555, Factor = 1).
    const size_t off = (size_t)job.proj * W * H;
    const float y = job.dual ? job.dual[k] : 0.0f;
    const float p = __ldg(job.meas + off + k);
    const float c = (float)(1.0f * p - 1.0f * value - y) / (float)(1.0f * len + 1.0f);
    job.corr[k] = c;
    if (job.dual) job.dual[k] = (float)((double)y + alpha * (double)c);
  }
}

template <class View>
__global__ void __launch_bounds__(128) fp_kernel(const ProjGeom *__restrict__ geom, const FpJob *__restrict__ jobs,
                                                 int nx, int ny, int nz, int W, int H, float sd, double alpha) {
  int i, j;
  tile_pixel(i, j);
  if (i >= W || j >= H) return;
  const FpJob job = jobs[blockIdx.z];
  fp_pixel<View>(geom, job, nx, ny, nz, W, H, sd, alpha, i, j);
}

__global__ void __launch_bounds__(128) splat_kernel(const ProjGeom *__restrict__ geom,
                                                    const SplatJob *__restrict__ jobs, int nx, int ny, int nz, int W,
                                                    int H, float sd) {
  int i, j;
  tile_pixel(i, j);
  if (i >= W || j >= H) return;
  const SplatJob job = jobs[blockIdx.z];
  const ProjGeom &g = geom[job.proj];
  const int n[3] = {nx, ny, nz};
  float vz[4], vu[4], tn, tf;
  produce_ray(g, nx, ny, nz, (float)i, (float)j, vz, vu, tn, tf);
  if (!(tn < tf)) return;
  SplatSampler smp{nx, ny, nz, __ldg(job.corr + i + j * W), job.contrib, job.weight, 0.0f};
  cast_ray(smp, n, vz, vu, tn, tf, sd);
}

// ---------------------------------------------------------------------------
// Ray-driven matched backprojection with shared-memory accumulation
// (SingleScalarVolume.core.h:85-96,149-199: every forward-projection sample
// adds corr * w_k and w_k to its 8 trilinear taps).  A block's 128 rays (a
// 16 x 8 pixel tile) are nearly parallel, so at any distance t along them
// their samples lie in a small region.  The block marches its rays together
// through slabs of t (kSlab voxels deep): each slab's taps are first bounded
// (a pass over the slab's sample positions alone), then accumulated into a
// shared-memory window of that bounding box with shared atomics, and the
// window is flushed to the global sums with float4 atomic adds, one per
// aligned group of four voxels that received anything.  Taps outside the
// window's capacity go to global atomics directly, so any geometry is
// handled.  The sample sequence is the forward projector's, replayed by a
// resumable copy of cast_ray (same float operations in the same order).
// ---------------------------------------------------------------------------
namespace rbp {
constexpr int kCap = 4096;       // window cells (contributions + weights: 32 KB)
constexpr float kSlab = 6.0f;    // slab depth in t (voxel units)
constexpr int kThreads = 128;

// cast_ray as a generator: settle() advances to the next pending sample (or
// the end), peek() is that sample's t, take() returns its position.
struct March {
  float vz[3], vu[3], step[3], tnear, tfar, sd, t1, tb, t, p[3], tMax[3], tDelta[3];
  int mode;  // 0: first sample pending, 1: in a segment, 2: between segments, 3: done
  __device__ __forceinline__ void init(const int n[3], const float z[4], const float u[4], float tn, float tf,
                                       float s) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      vz[a] = z[a];
      vu[a] = u[a];
      step[a] = u[a] * s;
    }
    tnear = tn;
    tfar = tf;
    sd = s;
    t1 = tn;
    const float pos1[3] = {vz[0] + vu[0] * t1, vz[1] + vu[1] * t1, vz[2] + vu[2] * t1};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      p[a] = pos1[a];
      const int bs = n[a];
      tDelta[a] = 0.0f;
      if (vu[a] == 0.0f) {
        tMax[a] = tfar;
      } else if (vu[a] < 0.0f) {
        const int blk = ((int)ceilf(pos1[a] - 0.5f) - 1) / bs;
        tMax[a] = ((float)(blk * bs) + 0.5f - vz[a]) / vu[a];
        tDelta[a] = (float)(-(1 * bs)) / vu[a];
      } else {
        const int blk = ((int)floorf(pos1[a] - 0.5f)) / bs;
        tMax[a] = ((float)((blk + 1) * bs) + 0.5f - vz[a]) / vu[a];
        tDelta[a] = (float)(1 * bs) / vu[a];
      }
    }
    mode = 0;
  }
  __device__ __forceinline__ void settle() {
    for (;;) {
      if (mode == 0 || mode == 3) return;
      if (mode == 1) {
        if (t < tb) return;
        if (tMax[0] < tMax[1]) {
          if (tMax[0] < tMax[2]) tMax[0] += tDelta[0];
          else tMax[2] += tDelta[2];
        } else {
          if (tMax[1] < tMax[2]) tMax[1] += tDelta[1];
          else tMax[2] += tDelta[2];
        }
        t1 = tb;
        mode = 2;
      }
      if (!(t1 < tfar)) {
        mode = 3;
        return;
      }
      tb = mac_min(mac_min(tMax[0], tMax[1]), tMax[2]);
      if (tb > tfar) tb = tfar;
      t = ceilf((t1 - tnear) / sd) * sd + tnear;
      p[0] = vz[0] + vu[0] * t;
      p[1] = vz[1] + vu[1] * t;
      p[2] = vz[2] + vu[2] * t;
      mode = 1;
    }
  }
  __device__ __forceinline__ float peek() const { return mode == 0 ? tnear : mode == 1 ? t : INFINITY; }
  // the pending sample's position, then advance (call with peek() finite)
  __device__ __forceinline__ void take(float &x, float &y, float &z) {
    x = p[0];
    y = p[1];
    z = p[2];
    if (mode == 0) {
      mode = 2;
    } else {
      t += sd;
      p[0] += step[0];
      p[1] += step[1];
      p[2] += step[2];
    }
    settle();
  }
};

// The sampler's clamp-then-truncate cell of a position.
__device__ __forceinline__ void cell(float x, float y, float z, const int n[3], int &i, int &j, int &k, float &t0,
                                    float &t1, float &t2) {
  x = mac_max(mac_min(x, (float)(n[0] - 1)), 0.0f);
  y = mac_max(mac_min(y, (float)(n[1] - 1)), 0.0f);
  z = mac_max(mac_min(z, (float)(n[2] - 1)), 0.0f);
  i = (int)x;
  j = (int)y;
  k = (int)z;
  t0 = x - (float)i;
  t1 = y - (float)j;
  t2 = z - (float)k;
}
}  // namespace rbp

__global__ void __launch_bounds__(rbp::kThreads) bp_ray_kernel(const ProjGeom *__restrict__ geom,
                                                               const SplatJob *__restrict__ jobs, int nx, int ny,
                                                               int nz, int W, int H, float sd) {
  using namespace rbp;
  __shared__ __align__(16) float win_c[kCap];
  __shared__ __align__(16) float win_w[kCap];
  __shared__ int bb[6];
  __shared__ unsigned tstart;
  const int tid = threadIdx.x;
  int pi, pj;
  tile_pixel(pi, pj);
  const SplatJob job = jobs[blockIdx.z];
  const int n[3] = {nx, ny, nz};
  March m;
  m.mode = 3;
  float corr = 0.0f;
  if (pi < W && pj < H) {
    const ProjGeom &g = geom[job.proj];
    float vz[4], vu[4], tn, tf;
    produce_ray(g, nx, ny, nz, (float)pi, (float)pj, vz, vu, tn, tf);
    if (tn < tf) {
      m.init(n, vz, vu, tn, tf, sd);
      corr = __ldg(job.corr + pi + pj * W);
    }
  }
  for (int q = tid; q < kCap; q += kThreads) {
    win_c[q] = 0.0f;
    win_w[q] = 0.0f;
  }
  if (tid == 0) tstart = 0x7f800000u;  // +inf; t >= 0 so float order = bit order
  __syncthreads();
  if (m.mode != 3) atomicMin(&tstart, __float_as_uint(m.peek()));
  __syncthreads();
  if (tstart == 0x7f800000u) return;  // no ray of this tile meets the volume
  float T = __uint_as_float(tstart);
  const bool vec = (nx & 3) == 0 && ((reinterpret_cast<uintptr_t>(job.contrib) | reinterpret_cast<uintptr_t>(job.weight)) & 15) == 0;
  for (;;) {
    const float Tlo = T;
    T += kSlab;
    if (tid < 3) bb[tid] = 0x7fffffff;
    else if (tid < 6) bb[tid] = -1;
    __syncthreads();
    // the slab's cells: the ray segment t in [max(Tlo, next sample), min(T,
    // tfar)] bounds the sample positions up to the float recurrence's drift
    // (hundredths of a voxel); one cell of margin on each side covers it and
    // taps, and any tap outside the window still goes to a global atomic
    {
      int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {-1, -1, -1};
      const float tn = m.peek();
      if (tn < T) {
        const float ta = fmaxf(Tlo, tn), tb = fminf(T, m.tfar);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float pa = m.vz[a] + m.vu[a] * ta, pb = m.vz[a] + m.vu[a] * tb;
          const float mn = mac_max(mac_min(fminf(pa, pb), (float)(n[a] - 1)), 0.0f);
          const float mx = mac_max(mac_min(fmaxf(pa, pb), (float)(n[a] - 1)), 0.0f);
          lo[a] = max((int)mn - 1, 0);
          hi[a] = min((int)mx + 2, n[a] - 1);
        }
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
          lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
          hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
      }
      if ((tid & 31) == 0 && hi[0] >= 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          atomicMin(&bb[a], lo[a]);
          atomicMax(&bb[3 + a], hi[a]);
        }
      }
    }
    __syncthreads();
    const bool any = bb[3] >= 0;
    // the window: x from a multiple of 4 (aligned float4 flushes), clipped to kCap cells
    const int ox = bb[0] & ~3, oy = bb[1], oz = bb[2];
    const int wx = any ? ((bb[3] - ox + 1) + 3) & ~3 : 4;
    const int wy = any ? min(bb[4] - oy + 1, max(1, kCap / wx)) : 1;
    const int wz = any ? min(bb[5] - oz + 1, max(1, kCap / (wx * wy))) : 1;
    const bool fits = wx * wy <= kCap;
    // pass 2: accumulate
    while (m.peek() < T) {
      float x, y, z, t0, t1, t2;
      int ci, cj, ck;
      m.take(x, y, z);
      cell(x, y, z, n, ci, cj, ck, t0, t1, t2);
      const float M0 = 1.0f - t0, M1 = 1.0f - t1, M2 = 1.0f - t2;
      const float w[8] = {M0 * M1 * M2, t0 * M1 * M2, M0 * t1 * M2, t0 * t1 * M2,
                          M0 * M1 * t2, t0 * M1 * t2, M0 * t1 * t2, t0 * t1 * t2};
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int x2 = ci + (c & 1), y2 = cj + ((c >> 1) & 1), z2 = ck + ((c >> 2) & 1);
        if (x2 >= nx || y2 >= ny || z2 >= nz) continue;
        const int lx = x2 - ox, ly = y2 - oy, lz = z2 - oz;
        const float cw = corr * w[c];
        if (fits && (unsigned)lx < (unsigned)wx && (unsigned)ly < (unsigned)wy && (unsigned)lz < (unsigned)wz) {
          const int q = lx + wx * (ly + wy * lz);
          atomicAdd(win_c + q, cw);
          atomicAdd(win_w + q, w[c]);
        } else {
          const size_t id = (size_t)x2 + (size_t)nx * (y2 + (size_t)ny * z2);
          atomicAdd(job.contrib + id, cw);
          atomicAdd(job.weight + id, w[c]);
        }
      }
    }
    __syncthreads();
    // flush: aligned groups of 4 cells along x that received anything
    if (any && fits) {
      const int gx = wx >> 2, ngroups = gx * wy * wz;
      for (int q = tid; q < ngroups; q += kThreads) {
        const int qx = q % gx, qy = (q / gx) % wy, qz = q / (gx * wy);
        const int base = 4 * qx + wx * (qy + wy * qz);
        const float4 c4 = *reinterpret_cast<const float4 *>(win_c + base);
        const float4 w4 = *reinterpret_cast<const float4 *>(win_w + base);
        if (w4.x == 0.0f && w4.y == 0.0f && w4.z == 0.0f && w4.w == 0.0f && c4.x == 0.0f && c4.y == 0.0f &&
            c4.z == 0.0f && c4.w == 0.0f)
          continue;
        *reinterpret_cast<float4 *>(win_c + base) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        *reinterpret_cast<float4 *>(win_w + base) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const int x = ox + 4 * qx, y = oy + qy, z = oz + qz;
        const size_t id = (size_t)x + (size_t)nx * (y + (size_t)ny * z);
        if (vec && x + 3 < nx) {
          atomicAdd(reinterpret_cast<float4 *>(job.contrib + id), c4);
          atomicAdd(reinterpret_cast<float4 *>(job.weight + id), w4);
        } else {
          const float cs[4] = {c4.x, c4.y, c4.z, c4.w}, ws[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (x + e < nx && (ws[e] != 0.0f || cs[e] != 0.0f)) {
              atomicAdd(job.contrib + id + e, cs[e]);
              atomicAdd(job.weight + id + e, ws[e]);
            }
        }
      }
    }
    if (!__syncthreads_or(m.peek() < INFINITY)) break;
  }
}

__global__ void ray_update_kernel(const RayUpdJob *__restrict__ jobs, int zblocks, int nx, int ny, float alpha,
                                  float gmax) {
  const int jb = blockIdx.z / zblocks;
  const RayUpdJob job = jobs[jb];
  const int x = job.box[0] + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = job.box[2] + blockIdx.y * blockDim.y + threadIdx.y;
  const int z = job.box[4] + (blockIdx.z % zblocks) * blockDim.z + threadIdx.z;
  if (x >= job.box[1] || y >= job.box[3] || z >= job.box[5]) return;
  const size_t t = (size_t)x + (size_t)nx * (y + (size_t)ny * z);
  const float w = job.weight[t];
  if (!(w > 0.0f)) return;
  float v = job.vol[t] + alpha * (job.contrib[t] / w);
  v = v < 0.0f ? 0.0f : (v > gmax ? gmax : v);
  job.vol[t] = v;
}

__global__ void correction_kernel(int n, const float *__restrict__ meas, const float *__restrict__ img,
                                  const float *__restrict__ len, float *dual, double alpha, float *corr) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float y = dual ? dual[k] : 0.0f;
  const float c = (float)(1.0f * meas[k] - 1.0f * img[k] - y) / (float)(1.0f * len[k] + 1.0f);
  corr[k] = c;
  if (dual) dual[k] = (float)((double)y + alpha * (double)c);
}

// ---------------------------------------------------------------------------
// Voxel-driven bicubic backprojection (WaP_Tomo.cpp:208-222, 1557-1628 and
// 1294-1374).  One thread per voxel; the 16 taps come from the correction
// image, which every block of a launch shares (L1/L2 resident).
// ---------------------------------------------------------------------------

// cubicInterpolate evaluated as the reference does: the float differences
// p2-p0 and p1-p2 first, everything else in double (the literals are double).
__device__ __forceinline__ float cubic_exact(float p0, float p1, float p2, float p3, float x) {
  const double xd = x;
  const double inner = 3.0 * (double)(p1 - p2) + (double)p3 - (double)p0;
  const double mid = 2.0 * (double)p0 - 5.0 * (double)p1 + 4.0 * (double)p2 - (double)p3 + xd * inner;
  const double outer = (double)(p2 - p0) + xd * mid;
  return (float)((double)p1 + 0.5 * xd * outer);
}

// The same Catmull-Rom polynomial in FP32 with fused multiply-adds.
__device__ __forceinline__ float cubic_fast(float p0, float p1, float p2, float p3, float x) {
  const float inner = __fmaf_rn(3.0f, p1 - p2, p3 - p0);
  const float mid = __fmaf_rn(x, inner, __fmaf_rn(2.0f, p0, __fmaf_rn(-5.0f, p1, __fmaf_rn(4.0f, p2, -p3))));
  const float outer = __fmaf_rn(x, mid, p2 - p0);
  return __fmaf_rn(0.5f * x, outer, p1);
}

// Index <-> float conversions without the conversion instructions (on this
// part they issue to a low-rate pipe): exact for 0 <= i < 2^23, and for
// 0 <= v < 2^22 respectively, which the callers guarantee.
__device__ __forceinline__ float small_i2f(int i) { return __int_as_float(0x4B000000 | i) - 8388608.0f; }
// floor(v) as float, for 0 <= v < 2^22: v + 2^23 rounds to the nearest
// integer exactly, and one correction step gives the floor.
__device__ __forceinline__ float small_floor(float v) {
  const float r = (v + 8388608.0f) - 8388608.0f;
  return r > v ? r - 1.0f : r;
}
__device__ __forceinline__ int small_f2i(float fl) { return __float_as_int(fl + 8388608.0f) - 0x4B000000; }

// Scalars of a voxel-driven backprojection: the host passes halfW, halfH, ds
// and alpha in both precisions (the f suffixes are the float roundings;
// alphal = alpha - (float)alpha); float_ok says halfW, halfH and ds are exact
// floats, so that a single double operation rounded to float equals the float
// operation.
struct BpParams {
  int nx, ny, W, H;
  double halfW, halfH;
  float sdd;
  double ds;
  int float_ok;
  double alpha;
  float gmax, halfWf, halfHf, dsf, alphaf, alphal, wlim, hlim;
};

// One voxel (x, y, z) of a backprojection job.  The pixel test px < 2 || px >=
// W-2 on px = (int)_px is the same as !(2 <= _px < W-2) for every float _px
// (NaN included), and for _px inside that range (int)_px = floor(_px).
template <bool kExact, int kMode>
__device__ __forceinline__ void bp_voxel(const ProjGeom *__restrict__ geom, const BpParams &P, const BpJob &job, int x,
                                         int y, int z) {
  const ProjGeom &g = geom[job.proj];
  const int W = P.W;
  float det[4];
  mat4_vec(g.mvv2m, small_i2f(x), small_i2f(y), small_i2f(z), 1.0f, det);
  const float qx = (det[0] / det[2]) * P.sdd;
  const float qy = (det[1] / det[2]) * P.sdd;
  float _px, _py;
  if (P.float_ok) {
    _px = P.halfWf - qx;
    _py = P.halfHf - qy;
    _px = _px / P.dsf;
    _py = _py / P.dsf;
  } else {
    _px = (float)(P.halfW - (double)qx);
    _py = (float)(P.halfH - (double)qy);
    _px = (float)((double)_px / P.ds);
    _py = (float)((double)_py / P.ds);
  }
  if (!(_px >= 2.0f && _px < P.wlim && _py >= 2.0f && _py < P.hlim)) return;
  const float fx = small_floor(_px), fy = small_floor(_py);
  const int px = small_f2i(fx), py = small_f2i(fy);
  const float dx = _px - fx, dy = _py - fy;
  const float *__restrict__ pC = job.corr + py * W + px;
  float pv[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float *c = pC + (r - 1);
    pv[r][0] = __ldg(c - W);
    pv[r][1] = __ldg(c);
    pv[r][2] = __ldg(c + W);
    pv[r][3] = __ldg(c + 2 * W);
  }
  float arr[4], gv;
  if (kExact) {
    // The reference's double arithmetic: certified float-float where the
    // float result is certain (nearly always), the FP64 pipe otherwise.
    bool ok = true;
#pragma unroll
    for (int r = 0; r < 4; ++r) ok = bpc::cubic_cert(pv[r][0], pv[r][1], pv[r][2], pv[r][3], dy, &arr[r]) && ok;
    ok = ok && bpc::cubic_cert(arr[0], arr[1], arr[2], arr[3], dx, &gv);
    if (!ok) {
#pragma unroll
      for (int r = 0; r < 4; ++r) arr[r] = cubic_exact(pv[r][0], pv[r][1], pv[r][2], pv[r][3], dy);
      gv = cubic_exact(arr[0], arr[1], arr[2], arr[3], dx);
    }
  } else {
#pragma unroll
    for (int r = 0; r < 4; ++r) arr[r] = cubic_fast(pv[r][0], pv[r][1], pv[r][2], pv[r][3], dy);
    gv = cubic_fast(arr[0], arr[1], arr[2], arr[3], dx);
  }
  float *v = job.vol + (x + P.nx * (y + P.ny * z));
  if (kMode == 0) {
    float nv;
    if (kExact) {
      if (!bpc::update_cert(*v, gv, P.alphaf, P.alphal, &nv)) nv = (float)((double)*v + P.alpha * (double)gv);
    } else {
      nv = __fmaf_rn(P.alphaf, gv, *v);
    }
    nv = mac_max(mac_min(P.gmax, nv), 0.0f);
    *v = nv;
  } else {
    *v = *v + gv;
  }
}

template <bool kExact, int kMode>
__global__ void __launch_bounds__(256) bp_voxel_kernel(const ProjGeom *__restrict__ geom,
                                                       const BpJob *__restrict__ jobs, int zblocks, BpParams P) {
  const int jb = blockIdx.z / zblocks;
  const BpJob job = jobs[jb];
  const int x = job.box[0] + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = job.box[2] + blockIdx.y * blockDim.y + threadIdx.y;
  const int z = job.box[4] + (blockIdx.z % zblocks) * blockDim.z + threadIdx.z;
  if (x >= job.box[1] || y >= job.box[3] || z >= job.box[5]) return;
  bp_voxel<kExact, kMode>(geom, P, job, x, y, z);
}

BpParams bp_params(const int dims[3], int W, int H, double halfW, double halfH, float sdd, double ds, double alpha,
                   float gmax) {
  BpParams P;
  P.nx = dims[0];
  P.ny = dims[1];
  P.W = W;
  P.H = H;
  P.halfW = halfW;
  P.halfH = halfH;
  P.sdd = sdd;
  P.ds = ds;
  P.float_ok = ((double)(float)halfW == halfW && (double)(float)halfH == halfH && (double)(float)ds == ds);
  P.alpha = alpha;
  P.gmax = gmax;
  P.halfWf = (float)halfW;
  P.halfHf = (float)halfH;
  P.dsf = (float)ds;
  P.alphaf = (float)alpha;
  P.alphal = (float)(alpha - (double)(float)alpha);  // alpha ~ (float)alpha + alphal
  P.wlim = (float)(W - 2);
  P.hlim = (float)(H - 2);
  return P;
}

// ---------------------------------------------------------------------------
// Work-queue kernels (wap_internal.h): persistent blocks take items from a
// counter; an item is one job's pixel tile / voxel block / brick tile, the
// job found by binary search over the jobs' first items.  No block waits on
// another, and the per-pixel / per-voxel code is the per-launch kernels'.
// ---------------------------------------------------------------------------
template <class J>
__device__ __forceinline__ int queue_job(const J *__restrict__ jobs, int njobs, int item) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].item0 <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// The next item for the whole block (uniform across its threads).
__device__ __forceinline__ int queue_next(int *counter, int *slot) {
  __syncthreads();  // every thread has read the previous item
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) *slot = atomicAdd(counter, 1);
  __syncthreads();
  return *slot;
}

// WX x WY warps, each an 8x4 pixel patch: a tile of 8 WX x 4 WY pixels.
template <int WX, int WY>
__global__ void __launch_bounds__(32 * WX * WY) fp_queue_kernel(const QFpJob *__restrict__ jobs, int njobs, int total,
                                                                int *counter) {
  __shared__ int slot;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  for (;;) {
    const int item = queue_next(counter, &slot);
    if (item >= total) return;
    const QFpJob &q = jobs[queue_job(jobs, njobs, item)];
    const int t = item - q.item0, tx = t % q.tiles_x, ty = t / q.tiles_x;
    const int i = tx * (8 * WX) + (w % WX) * 8 + (lane & 7);
    const int j = ty * (4 * WY) + (w / WX) * 4 + (lane >> 3);
    if (i >= q.W || j >= q.H) continue;
    if (q.bricked == 2)
      fp_pixel<BrickViewH>(q.geom, q.job, q.n[0], q.n[1], q.n[2], q.W, q.H, q.sd, q.alpha, i, j);
    else if (q.bricked)
      fp_pixel<BrickView>(q.geom, q.job, q.n[0], q.n[1], q.n[2], q.W, q.H, q.sd, q.alpha, i, j);
    else
      fp_pixel<VolView>(q.geom, q.job, q.n[0], q.n[1], q.n[2], q.W, q.H, q.sd, q.alpha, i, j);
  }
}

template <bool kExact, int kMode, int BX, int BY, int BZ>
__global__ void __launch_bounds__(BX * BY * BZ) bp_queue_kernel(const QBpJob *__restrict__ jobs, int njobs,
                                                                int total, int *counter) {
  __shared__ int slot;
  const int tx = threadIdx.x % BX, ty = (threadIdx.x / BX) % BY, tz = threadIdx.x / (BX * BY);
  for (;;) {
    const int item = queue_next(counter, &slot);
    if (item >= total) return;
    const QBpJob &q = jobs[queue_job(jobs, njobs, item)];
    const int t = item - q.item0;
    const int bx = t % q.bx, by = (t / q.bx) % q.by, bz = t / (q.bx * q.by);
    const int x = q.job.box[0] + bx * BX + tx, y = q.job.box[2] + by * BY + ty, z = q.job.box[4] + bz * BZ + tz;
    if (x >= q.job.box[1] || y >= q.job.box[3] || z >= q.job.box[5]) continue;
    const BpParams P = *reinterpret_cast<const BpParams *>(&q.P);
    bp_voxel<kExact, kMode>(q.geom, P, q.job, x, y, z);
  }
}

__global__ void __launch_bounds__(256) brick_queue_kernel(const QBrickJob *__restrict__ jobs, int njobs, int total,
                                                          int *counter) {
  __shared__ float t[4][4][32];
  __shared__ int slot;
  for (;;) {
    const int item = queue_next(counter, &slot);
    if (item >= total) return;
    const QBrickJob &q = jobs[queue_job(jobs, njobs, item)];
    const int r = item - q.item0, bx = r % q.tx, by = (r / q.tx) % q.ty, bz = r / (q.tx * q.ty);
    if (q.half)
      brick_tile(q.vol, reinterpret_cast<__half *>(q.out), q.n[0], q.n[1], q.n[2], bx * 32, by * 4, bz * 4, t);
    else
      brick_tile(q.vol, q.out, q.n[0], q.n[1], q.n[2], bx * 32, by * 4, bz * 4, t);
  }
}

template <class K>
int resident_blocks(K kernel, int threads) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0) != cudaSuccess || per < 1) per = 1;
  return per;
}
int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
  }
  return n;
}

// Resident blocks per SM of every work-queue kernel, asked once (so no
// occupancy query runs while a graph is being captured: warm_queue_kernels).
struct QueueOcc {
  int fp[kFpShapes], bp[2][2][kBpShapes], brick;
};
const QueueOcc &queue_occ() {
  static const QueueOcc occ = [] {
    QueueOcc q;
    q.fp[0] = resident_blocks(fp_queue_kernel<2, 2>, 128);
    q.fp[1] = resident_blocks(fp_queue_kernel<1, 2>, 64);
    q.fp[2] = resident_blocks(fp_queue_kernel<4, 2>, 256);
#define WAP_OCC(E, M)                                                    \
  q.bp[E][M][0] = resident_blocks(bp_queue_kernel<E, M, 32, 4, 2>, 256); \
  q.bp[E][M][1] = resident_blocks(bp_queue_kernel<E, M, 32, 8, 1>, 256); \
  q.bp[E][M][2] = resident_blocks(bp_queue_kernel<E, M, 32, 2, 4>, 256);
    WAP_OCC(false, 0)
    WAP_OCC(false, 1)
    WAP_OCC(true, 0)
    WAP_OCC(true, 1)
#undef WAP_OCC
    q.brick = resident_blocks(brick_queue_kernel, 256);
    return q;
  }();
  return occ;
}

}  // namespace

static_assert(sizeof(QBpParams) == sizeof(BpParams), "the host's QBpParams mirrors BpParams");

void warm_queue_kernels() {
  (void)queue_occ();
  (void)sm_count();
}

QBpParams make_bp_params(const int dims[3], int W, int H, double halfW, double halfH, float sdd, double ds,
                         double alpha, float gmax) {
  const BpParams P = bp_params(dims, W, H, halfW, halfH, sdd, ds, alpha, gmax);
  QBpParams Q;
  std::memcpy(&Q, &P, sizeof(Q));
  return Q;
}

void fp_shape_tile(int shape, int &tw, int &th) {
  tw = shape == 1 ? 8 : shape == 2 ? 32 : 16;
  th = 8;
}
void bp_shape_block(int shape, int &bx, int &by, int &bz) {
  bx = 32;
  by = shape == 1 ? 8 : shape == 2 ? 2 : 4;
  bz = shape == 1 ? 1 : shape == 2 ? 4 : 2;
}

int fp_queue_items(QFpJob *h, int njobs, int shape) {
  int tw, th, total = 0;
  fp_shape_tile(shape, tw, th);
  for (int j = 0; j < njobs; ++j) {
    h[j].tiles_x = (h[j].W + tw - 1) / tw;
    h[j].item0 = total;
    total += h[j].tiles_x * ((h[j].H + th - 1) / th);
  }
  return total;
}
int bp_queue_items(QBpJob *h, int njobs, int shape) {
  int bx, by, bz, total = 0;
  bp_shape_block(shape, bx, by, bz);
  for (int j = 0; j < njobs; ++j) {
    const int *b = h[j].job.box;
    const int ex = std::max(0, b[1] - b[0]), ey = std::max(0, b[3] - b[2]), ez = std::max(0, b[5] - b[4]);
    h[j].bx = (ex + bx - 1) / bx;
    h[j].by = (ey + by - 1) / by;
    h[j].item0 = total;
    total += h[j].bx * h[j].by * ((ez + bz - 1) / bz);
  }
  return total;
}
int brick_queue_items(QBrickJob *h, int njobs) {
  int total = 0;
  for (int j = 0; j < njobs; ++j) {
    h[j].tx = (h[j].n[0] + 31) / 32;
    h[j].ty = (h[j].n[1] + 3) / 4;
    h[j].item0 = total;
    total += h[j].tx * h[j].ty * ((h[j].n[2] + 3) / 4);
  }
  return total;
}

cudaError_t launch_fp_queue(const QFpJob *d_jobs, int njobs, int total, int *d_counter, int shape, cudaStream_t st) {
  if (njobs <= 0 || total <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  const int g = std::min(total, queue_occ().fp[shape == 1 || shape == 2 ? shape : 0] * sm_count());
  if (shape == 1) fp_queue_kernel<1, 2><<<g, 64, 0, st>>>(d_jobs, njobs, total, d_counter);
  else if (shape == 2) fp_queue_kernel<4, 2><<<g, 256, 0, st>>>(d_jobs, njobs, total, d_counter);
  else fp_queue_kernel<2, 2><<<g, 128, 0, st>>>(d_jobs, njobs, total, d_counter);
  return cudaGetLastError();
}

cudaError_t launch_bp_queue(const QBpJob *d_jobs, int njobs, int total, int *d_counter, int shape, int exact,
                            int mode, cudaStream_t st) {
  if (njobs <= 0 || total <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  const int sh = shape == 1 || shape == 2 ? shape : 0;
  const int g = std::min(total, queue_occ().bp[exact ? 1 : 0][mode ? 1 : 0][sh] * sm_count());
#define WAP_BPQ(E, M, BX, BY, BZ) \
  bp_queue_kernel<E, M, BX, BY, BZ><<<g, BX * BY * BZ, 0, st>>>(d_jobs, njobs, total, d_counter);
#define WAP_BPQ_SHAPE(E, M)                    \
  if (sh == 1) WAP_BPQ(E, M, 32, 8, 1)         \
  else if (sh == 2) WAP_BPQ(E, M, 32, 2, 4)    \
  else WAP_BPQ(E, M, 32, 4, 2)
  if (exact) {
    if (mode == 0) WAP_BPQ_SHAPE(true, 0)
    else WAP_BPQ_SHAPE(true, 1)
  } else {
    if (mode == 0) WAP_BPQ_SHAPE(false, 0)
    else WAP_BPQ_SHAPE(false, 1)
  }
#undef WAP_BPQ_SHAPE
#undef WAP_BPQ
  return cudaGetLastError();
}

cudaError_t launch_brick_queue(const QBrickJob *d_jobs, int njobs, int total, int *d_counter, cudaStream_t st) {
  if (njobs <= 0 || total <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  brick_queue_kernel<<<std::min(total, queue_occ().brick * sm_count()), 256, 0, st>>>(d_jobs, njobs, total,
                                                                                     d_counter);
  return cudaGetLastError();
}

cudaError_t launch_forward(const ProjGeom *d_geom, const FpJob *d_jobs, int njobs, const int dims[3], int W, int H,
                           float sd, double alpha, cudaStream_t st, bool bricked, bool half) {
  if (njobs <= 0) return cudaSuccess;
  dim3 grid((W + 15) / 16, (H + 7) / 8, njobs);
  if (bricked && half)
    fp_kernel<BrickViewH><<<grid, 128, 0, st>>>(d_geom, d_jobs, dims[0], dims[1], dims[2], W, H, sd, alpha);
  else if (bricked) fp_kernel<BrickView><<<grid, 128, 0, st>>>(d_geom, d_jobs, dims[0], dims[1], dims[2], W, H, sd, alpha);
  else fp_kernel<VolView><<<grid, 128, 0, st>>>(d_geom, d_jobs, dims[0], dims[1], dims[2], W, H, sd, alpha);
  return cudaGetLastError();
}

size_t brick_floats(const int dims[3]) {
  return (size_t)((dims[0] + 3) >> 2) * ((dims[1] + 3) >> 2) * ((dims[2] + 3) >> 2) * 64;
}

cudaError_t launch_brick_jobs(const FpJob *d_jobs, int njobs, float *out, const int dims[3], cudaStream_t st,
                              bool half) {
  if ((size_t)dims[0] * dims[1] * dims[2] == 0 || njobs <= 0) return cudaSuccess;
  const int ztiles = (dims[2] + 3) / 4;
  if ((long long)ztiles * njobs > 65535 || (dims[1] + 3) / 4 > 65535) return cudaErrorInvalidValue;
  const dim3 g((unsigned)((dims[0] + 31) / 32), (unsigned)((dims[1] + 3) / 4), (unsigned)(ztiles * njobs));
  // the FP16 copies start where the FP32 slots do (brick_floats(dims) floats,
  // twice as many halves, apart) and fill half of each
  if (half)
    brick_jobs_kernel<__half><<<g, 256, 0, st>>>(d_jobs, reinterpret_cast<__half *>(out), 2 * brick_floats(dims),
                                                 dims[0], dims[1], dims[2], ztiles);
  else
    brick_jobs_kernel<float><<<g, 256, 0, st>>>(d_jobs, out, brick_floats(dims), dims[0], dims[1], dims[2], ztiles);
  return cudaGetLastError();
}

cudaError_t launch_brick(const float *vol, float *out, const int dims[3], cudaStream_t st) {
  if ((size_t)dims[0] * dims[1] * dims[2] == 0) return cudaSuccess;
  if ((dims[2] + 3) / 4 > 65535 || (dims[1] + 3) / 4 > 65535) return cudaErrorInvalidValue;
  const dim3 g((unsigned)((dims[0] + 31) / 32), (unsigned)((dims[1] + 3) / 4), (unsigned)((dims[2] + 3) / 4));
  brick_kernel<<<g, 256, 0, st>>>(vol, out, dims[0], dims[1], dims[2]);
  return cudaGetLastError();
}

cudaError_t launch_ray_update(const RayUpdJob *d_jobs, int njobs, const int maxbox[3], const int dims[3],
                              double alpha, float gmax, cudaStream_t st) {
  if (njobs <= 0 || maxbox[0] <= 0 || maxbox[1] <= 0 || maxbox[2] <= 0) return cudaSuccess;
  const dim3 block(32, 4, 2);
  const int zblocks = (maxbox[2] + 1) / 2;
  if ((long long)zblocks * njobs > 65535) return cudaErrorInvalidValue;
  const dim3 grid((maxbox[0] + 31) / 32, (maxbox[1] + 3) / 4, zblocks * njobs);
  ray_update_kernel<<<grid, block, 0, st>>>(d_jobs, zblocks, dims[0], dims[1], (float)alpha, gmax);
  return cudaGetLastError();
}

cudaError_t launch_ray_splat(const ProjGeom *d_geom, const SplatJob *d_jobs, int njobs, const int dims[3], int W,
                             int H, float sd, cudaStream_t st, bool direct) {
  if (njobs <= 0) return cudaSuccess;
  dim3 grid((W + 15) / 16, (H + 7) / 8, njobs);
  if (direct) splat_kernel<<<grid, 128, 0, st>>>(d_geom, d_jobs, dims[0], dims[1], dims[2], W, H, sd);
  else bp_ray_kernel<<<grid, rbp::kThreads, 0, st>>>(d_geom, d_jobs, dims[0], dims[1], dims[2], W, H, sd);
  return cudaGetLastError();
}

cudaError_t launch_correction(int n, const float *meas, const float *img, const float *len, float *dual,
                              double alpha, float *corr, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  correction_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, meas, img, len, dual, alpha, corr);
  return cudaGetLastError();
}

cudaError_t launch_bp_voxel(const ProjGeom *d_geom, const BpJob *d_jobs, int njobs, int maxbox[3], const int dims[3],
                            int W, int H, double halfW, double halfH, float sdd, double ds, double alpha, float gmax,
                            int mode, int exact, cudaStream_t st) {
  if (njobs <= 0 || maxbox[0] <= 0 || maxbox[1] <= 0 || maxbox[2] <= 0) return cudaSuccess;
  const dim3 block(32, 4, 2);
  const int zblocks = (maxbox[2] + 1) / 2;
  const dim3 grid((maxbox[0] + 31) / 32, (maxbox[1] + 3) / 4, zblocks * njobs);
  if (W >= (1 << 22) || H >= (1 << 22)) return cudaErrorInvalidValue;
  const BpParams P = bp_params(dims, W, H, halfW, halfH, sdd, ds, alpha, gmax);
#define WAP_BP(E, M) bp_voxel_kernel<E, M><<<grid, block, 0, st>>>(d_geom, d_jobs, zblocks, P)
  if (exact) {
    if (mode == 0) WAP_BP(true, 0);
    else WAP_BP(true, 1);
  } else {
    if (mode == 0) WAP_BP(false, 0);
    else WAP_BP(false, 1);
  }
#undef WAP_BP
  return cudaGetLastError();
}

}  // namespace wap

namespace wap {
namespace {
__global__ void max_reduce_kernel(const float *__restrict__ d, size_t n, unsigned *out_bits) {
  // Non-negative-agnostic max via ordered integer keys.
  float m = -3.4028234663852886e38f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = fmaxf(m, d[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) {
    unsigned b = __float_as_uint(m);
    b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    atomicMax(out_bits, b);
  }
}
}  // namespace

cudaError_t launch_max_reduce(const float *d, size_t n, unsigned *d_bits, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(d_bits, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  max_reduce_kernel<<<152, 256, 0, st>>>(d, n, d_bits);
  return cudaGetLastError();
}

float decode_max_bits(unsigned b) {
  b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
  float f;
  memcpy(&f, &b, 4);
  return f;
}

}  // namespace wap
