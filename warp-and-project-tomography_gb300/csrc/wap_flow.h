// Flow-solver and CP-prior kernel interfaces (flow.cu, cp_prior.cu).
#pragma once

#include <cmath>
#include <vector>

#include "wap_internal.h"

namespace wap {

struct FlowDims {
  int n[3];
  int roi[6];  // margins: x-lo, x-hi, y-lo, y-hi, z-lo, z-hi (optical_flow.h ROI)
};

struct DericheCoefs {
  float a0, a1, a2, a3, b1, b2, coefp, coefn;
  int skip;  // sigma < 0.1: the filter is the identity
};

// Per-axis resize tables (device pointers).  Shrinking uses taps, growing uses
// base index + fractional offset accumulated in double as CImg does.
struct ResizeTables {
  const int *tap_start = nullptr;  // Sout + 1
  const int *tap_src = nullptr;
  const float *tap_w = nullptr;
  const int *base = nullptr;       // Sout
  const double *frac = nullptr;    // 3 * Sout: t, t*t, t*t*t per output cell
  const float *frac_ff = nullptr;  // 6 * Sout: each of those as a float pair hi + lo
};

DericheCoefs deriche_coefs(float sigma);
cudaError_t launch_deriche(int axis, const int dims[3], int nc, const DericheCoefs &k, const float *in, float *out,
                           cudaStream_t st);
// fast: growth in float with fused multiply-adds (the precision form); false:
// CImg's double cubic, bit for bit.
cudaError_t launch_resize_axis(int axis, const int in_dims[3], int nc, int Sout, const ResizeTables &tb,
                               const float *in, float *out, cudaStream_t st, bool fast = false);
cudaError_t launch_linearize(const FlowDims &D, const float *warp, const float *I1, const float *v, float *u,
                             float *kx4prev, cudaStream_t st);
cudaError_t launch_pd_fused(const FlowDims &D, int zchunk, const float *yin, float *yout, const float *u,
                            const float *vin, float *vout, float *kty, const float *kx4prev, int kxold_mode,
                            float lambda, float sigma1, float rinv, int fastdiv, int rcp, int store_kty, int residual,
                            double *acc, cudaStream_t st);
// The same iteration as two kernels (primal, then dual); identical results.
// rcp = 1 computes 1/x with the verified fast reciprocal.
cudaError_t launch_pd_split(const FlowDims &D, int zchunk, const float *yin, float *yout, const float *u,
                            const float *vin, float *vout, float *kty, const float *kx4prev, int kxold_mode,
                            float lambda, float sigma1, float rinv, int fastdiv, int rcp, int store_kty,
                            int residual, double *acc, cudaStream_t st);
// The TMA-fed fused form (nx % 4 == 0).  Tensor maps (64-byte opaque
// descriptors, 64-byte aligned storage) over y (10 ch), u (4 ch), v (3 ch).
struct alignas(64) PdTmaMap {
  unsigned char bytes[128];
};
// half = the precision form: y, u, v stored as FP16 pairs with the fast FP32
// arithmetic; otherwise FP32 storage, exact.  Both need nx % 4 == 0.
bool pd_tma_supported(const FlowDims &D, bool half);
// Blocks of the TMA form resident on the whole GPU at once (SMs x blocks per
// SM; 0 if the query fails) and the (x, y) tiles of a grid: a z-chunk count
// making tiles x chunks a multiple of the slots fills whole waves.
int pd_tma_slots(bool half);
int pd_tma_tiles(const FlowDims &D);
cudaError_t make_pd_tma_maps(const FlowDims &D, bool half, const void *y, const void *u, const void *v, void *ymap,
                             void *umap, void *vmap);
cudaError_t launch_pd_tma(const FlowDims &D, int zchunk, bool half, const void *ymap, const void *umap,
                          const void *vmap, void *yout, void *vout, float *kty, const float *kx4prev, int kxold_mode,
                          float lambda, float sigma1, float rinv, int fastdiv, int rcp, int store_kty, int residual,
                          double *acc, int *err, cudaStream_t st);
// nc component planes of nv floats <-> ceil(nc/2) planes of FP16 pairs
// (components 2q and 2q+1 in one 32-bit word, an odd last one paired with 0;
// round to nearest even), the precision form's storage.
cudaError_t launch_to_pairs(size_t nv, int nc, const float *src, void *dst, cudaStream_t st);
cudaError_t launch_from_pairs(size_t nv, int nc, const void *src, float *dst, cudaStream_t st);
// Counts the float inputs for which the FMA-corrected division by den differs
// from IEEE division (0 proves the fast path exact for this den).
cudaError_t launch_pd_fastdiv_check(float den, float rinv, unsigned long long *d_bad, cudaStream_t st);
// Counts the float inputs for which the fast reciprocal differs from 1.0f / x.
cudaError_t launch_pd_rcp_check(unsigned long long *d_bad, cudaStream_t st);
cudaError_t launch_residual_finish(const double *acc, int nPx, float *err, cudaStream_t st);
cudaError_t launch_roi_copy(const FlowDims &D, int nch, const float *src, float *dst, cudaStream_t st);

// CP prior (WaP_Tomo.cpp:586-689), batched over frames.
struct CpArgs {
  int n[3];
  int box[6];
  int f0;          // first frame of the batch
  int F;           // frames in the batch
  int Ftot;        // frames in the level (X_bar[Ftot] is the zero volume)
  float sigma;     // CP_sigma = .9/(L*tau)
  float tau;       // CP_tau
  float tv_w, tp_w;
  float gmax;
};
cudaError_t launch_cp_dual(const CpArgs &a, const float *xbar, const float *xbar_zero, float *ytv, float *ytp,
                           cudaStream_t st);
cudaError_t launch_cp_primal(const CpArgs &a, const float *ytp, const float *ytv, float *vol, float *xprev,
                             cudaStream_t st);
cudaError_t launch_cp_overrelax(const CpArgs &a, const float *vol, const float *xprev, float *xbar, cudaStream_t st);

// Host-side table builders for the resize kernels.
struct HostResizeAxis {
  std::vector<int> tap_start, tap_src, base;
  std::vector<float> tap_w;
  std::vector<double> frac;
};
HostResizeAxis make_resize_axis(int Sin, int Sout);

}  // namespace wap
