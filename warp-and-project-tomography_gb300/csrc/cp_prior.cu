// Chambolle-Pock spatial-TV / temporal prior of PSART::Render
// (WaP_Tomo.cpp:586-689), batched over all frames of a time level.
//
// Within one CP iteration every frame's dual reads only the previous
// iteration's over-relaxed volumes X_bar[f] and X_bar[f+1], and frame f's
// primal reads Y_tp[f-1] and Y_tp[f] of the current iteration, so the
// reference's frame loop splits into three frame-parallel launches around
// the (frame-parallel) SART sweeps: dual(all) -> primal(all) -> SART(all) ->
// over-relaxation(all).  Only channel 0 of the reference's 3-channel Y_tp /
// X_bar is ever read and Y_bc stays zero, so they are one channel here.
#include <algorithm>

#include "wap_flow.h"

namespace wap {
namespace {

__global__ void cp_dual_kernel(CpArgs a, const float *__restrict__ xbar, const float *__restrict__ xbar_zero,
                               float *__restrict__ ytv, float *__restrict__ ytp) {
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z % nz;
  const int f = a.f0 + (int)(blockIdx.z / nz);
  if (i >= nx || j >= ny) return;
  const size_t nv = (size_t)nx * ny * nz;
  const size_t t = i + (size_t)nx * (j + (size_t)ny * k);
  const float *xb = xbar + f * nv;
  const float *xn = (f + 1 < a.Ftot) ? xbar + (f + 1) * nv : xbar_zero;
  float *tp = ytp + f * nv;
  // Y_tp[f] += sigma * (X_bar[f+1] - X_bar[f]) over all voxels.
  float yp = tp[t] + (xn[t] - xb[t]) * a.sigma;
  const bool in_box = i >= a.box[0] && i < a.box[1] && j >= a.box[2] && j < a.box[3] && k >= a.box[4] && k < a.box[5];
  if (in_box) {
    float *tv = ytv + 3 * f * nv;
    const float x0 = xb[t];
    const float d[3] = {xb[t + 1] - x0, xb[t + nx] - x0, xb[t + (size_t)nx * ny] - x0};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float y = tv[c * nv + t] + a.sigma * d[c] * 1.0f;
      y = mac_max(-a.tv_w, mac_min(a.tv_w, y));
      tv[c * nv + t] = y;
    }
    yp = yp * a.tp_w / (a.tp_w + 2 * a.sigma);
  }
  tp[t] = yp;
}

__global__ void cp_primal_kernel(CpArgs a, const float *__restrict__ ytp, const float *__restrict__ ytv,
                                 float *__restrict__ vol, float *__restrict__ xprev) {
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z % nz;
  const int f = a.f0 + (int)(blockIdx.z / nz);
  if (i >= nx || j >= ny) return;
  const size_t nv = (size_t)nx * ny * nz;
  const size_t t = i + (size_t)nx * (j + (size_t)ny * k);
  float *v = vol + f * nv;
  float x = v[t];
  xprev[f * nv + t] = x;
  // Temporal primal term over all voxels (WaP_Tomo.cpp:626-639).
  const float *tp = ytp + f * nv;
  if (f == 0) x = x - (0.0f - tp[t]) * a.tau;
  else x = x - (tp[t - nv] - tp[t]) * a.tau;
  const bool in_box = i >= a.box[0] && i < a.box[1] && j >= a.box[2] && j < a.box[3] && k >= a.box[4] && k < a.box[5];
  if (in_box) {
    const float *tv = ytv + 3 * f * nv;
    const size_t sxy = (size_t)nx * ny;
    const float y1 = -(tv[t] - tv[t - 1] + tv[nv + t] - tv[nv + t - nx] + tv[2 * nv + t] - tv[2 * nv + t - sxy]);
    x -= (a.tau * y1);
    x = mac_max(mac_min(a.gmax, x), 0.0f);
  }
  v[t] = x;
}

__global__ void cp_overrelax_kernel(CpArgs a, const float *__restrict__ vol, const float *__restrict__ xprev,
                                    float *__restrict__ xbar) {
  const int nx = a.n[0], ny = a.n[1], nz = a.n[2];
  const int i = a.box[0] + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = a.box[2] + blockIdx.y * blockDim.y + threadIdx.y;
  const int bz = a.box[5] - a.box[4];
  const int k = a.box[4] + blockIdx.z % bz;
  const int f = a.f0 + (int)(blockIdx.z / bz);
  if (i >= a.box[1] || j >= a.box[3]) return;
  const size_t nv = (size_t)nx * ny * nz;
  const size_t t = f * nv + i + (size_t)nx * (j + (size_t)ny * k);
  xbar[t] = 2 * vol[t] - xprev[t];
}

}  // namespace

// The frames of a batch go in gridDim.z (z planes x frames); batches whose
// product would pass 65535 are split into several launches of whole frames.
// Each stage (dual, primal, over-relaxation) only reads what the previous
// stage wrote, so splitting a stage changes nothing.
template <class Launch>
cudaError_t for_frame_chunks(const CpArgs &a, int zplanes, Launch launch) {
  const int per = std::max(1, 65535 / std::max(1, zplanes));
  for (int f = 0; f < a.F; f += per) {
    CpArgs c = a;
    c.f0 = a.f0 + f;
    c.F = std::min(per, a.F - f);
    launch(c);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_cp_dual(const CpArgs &a, const float *xbar, const float *xbar_zero, float *ytv, float *ytp,
                           cudaStream_t st) {
  return for_frame_chunks(a, a.n[2], [&](const CpArgs &c) {
    const dim3 b(32, 8, 1), g((c.n[0] + 31) / 32, (c.n[1] + 7) / 8, c.n[2] * c.F);
    cp_dual_kernel<<<g, b, 0, st>>>(c, xbar, xbar_zero, ytv, ytp);
  });
}

cudaError_t launch_cp_primal(const CpArgs &a, const float *ytp, const float *ytv, float *vol, float *xprev,
                             cudaStream_t st) {
  return for_frame_chunks(a, a.n[2], [&](const CpArgs &c) {
    const dim3 b(32, 8, 1), g((c.n[0] + 31) / 32, (c.n[1] + 7) / 8, c.n[2] * c.F);
    cp_primal_kernel<<<g, b, 0, st>>>(c, ytp, ytv, vol, xprev);
  });
}

cudaError_t launch_cp_overrelax(const CpArgs &a, const float *vol, const float *xprev, float *xbar, cudaStream_t st) {
  const int bx = a.box[1] - a.box[0], by = a.box[3] - a.box[2], bz = a.box[5] - a.box[4];
  if (bx <= 0 || by <= 0 || bz <= 0) return cudaSuccess;
  return for_frame_chunks(a, bz, [&](const CpArgs &c) {
    const dim3 b(32, 8, 1), g((bx + 31) / 32, (by + 7) / 8, bz * c.F);
    cp_overrelax_kernel<<<g, b, 0, st>>>(c, vol, xprev, xbar);
  });
}

}  // namespace wap
