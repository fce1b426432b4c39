// Conjugate gradients on a volume (image_cg::cg, cg.h:11-55, with the
// image_blas vector operations of image_blas.h:9-91).  cg.h has no caller in
// the reference; the operator here is the SPD screened Laplacian
// A x = a x - b (sum of the 6 clamped neighbours - 6 x), the system the
// reference's test-free CG would be pointed at.  Vectors are FP32; every dot
// product is a warp-shuffle reduction accumulated in FP64, and the scalar
// recurrences (alpha, beta, the convergence ratio) stay on the device.
#include <cmath>

#include "wap/wap.h"
#include "wap_internal.h"

namespace wap {
namespace {

__device__ __forceinline__ void add_block_sum(double v, double *dst) {
  __shared__ double sh[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int tid = threadIdx.x;
  if ((tid & 31) == 0) sh[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) s += sh[w];
    atomicAdd(dst, s);
  }
}

struct Lap {
  int nx, ny, nz;
  float a, b;
};

// out = A in; acc += dot(in, out)
__global__ void lap_apply_kernel(Lap L, const float *__restrict__ in, float *__restrict__ out, double *acc) {
  const size_t n = (size_t)L.nx * L.ny * L.nz;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double part = 0.0;
  if (t < n) {
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((size_t)L.nx * L.ny));
    const size_t sy = L.nx, sz = (size_t)L.nx * L.ny;
    const float xc = in[t];
    const float s = in[i > 0 ? t - 1 : t] + in[i < L.nx - 1 ? t + 1 : t] + in[j > 0 ? t - sy : t] +
                    in[j < L.ny - 1 ? t + sy : t] + in[k > 0 ? t - sz : t] + in[k < L.nz - 1 ? t + sz : t];
    const float y = L.a * xc - L.b * (s - 6.0f * xc);
    out[t] = y;
    part = (double)xc * (double)y;
  }
  if (acc) add_block_sum(part, acc);
}

// r = b - Ap, p = r, acc += dot(r, r)
__global__ void cg_init_kernel(size_t n, const float *__restrict__ rhs, const float *__restrict__ ap,
                               float *__restrict__ r, float *__restrict__ p, double *acc) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double part = 0.0;
  if (t < n) {
    const float rv = (float)((double)rhs[t] + (double)ap[t] * -1.0);
    r[t] = rv;
    p[t] = rv;
    part = (double)rv * (double)rv;
  }
  add_block_sum(part, acc);
}

// scal[0] = rr_old, scal[1] = alpha; sums[] are the FP64 accumulators.
__global__ void cg_alpha_kernel(const double *__restrict__ pap, float *__restrict__ scal) {
  scal[1] = scal[0] / (float)pap[0];
}

// x += alpha p; r += (-alpha) Ap; acc += dot(r, r)
__global__ void cg_update_kernel(size_t n, const float *__restrict__ scal, const float *__restrict__ p,
                                 const float *__restrict__ ap, float *__restrict__ x, float *__restrict__ r,
                                 double *acc) {
  const float alpha = scal[1];
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double part = 0.0;
  if (t < n) {
    x[t] = x[t] + p[t] * alpha;
    const float rv = r[t] + ap[t] * -alpha;
    r[t] = rv;
    part = (double)rv * (double)rv;
  }
  add_block_sum(part, acc);
}

// p = r + beta p (mode 0) or p = r + 0 * beta (mode 1, the reference's aliasing).
__global__ void cg_direction_kernel(size_t n, const float *__restrict__ scal, const float *__restrict__ r,
                                    float *__restrict__ p, int mode) {
  const float beta = scal[2] / scal[0];
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  p[t] = mode == 1 ? r[t] + 0.0f * beta : r[t] + p[t] * beta;
}

__global__ void cg_store_rr_kernel(const double *__restrict__ acc, float *__restrict__ scal, int slot) {
  scal[slot] = (float)acc[0];
}

__global__ void cg_shift_rr_kernel(float *__restrict__ scal) { scal[0] = scal[2]; }

}  // namespace
}  // namespace wap

using namespace wap;

extern "C" int wap_cg_screened_laplacian(wap_ctx *ctx, const int *dims, float a, float b, const float *d_rhs,
                                         float *d_x, float rel_tol, int max_iters, float abs_tol, int mode,
                                         int *h_iters) {
  if (!ctx || !dims || !d_rhs || !d_x || dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || max_iters < 0)
    return WAP_EINVAL;
  cudaStream_t st = ctx_stream(ctx);
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  float *buf = nullptr;
  double *acc = nullptr;
  float *scal = nullptr;
  if (cudaMalloc(&buf, sizeof(float) * 3 * n) != cudaSuccess) return WAP_ENOMEM;
  if (cudaMalloc(&acc, sizeof(double) * 4) != cudaSuccess || cudaMalloc(&scal, sizeof(float) * 4) != cudaSuccess) {
    cudaFree(buf);
    cudaFree(acc);
    return WAP_ENOMEM;
  }
  float *r = buf, *p = buf + n, *ap = buf + 2 * n;
  const Lap L{dims[0], dims[1], dims[2], a, b};
  const unsigned blocks = (unsigned)((n + 255) / 256);
  int status = WAP_OK, iters = 0;
  auto check = [&]() {
    if (cudaGetLastError() != cudaSuccess) status = WAP_ECUDA;
    return status == WAP_OK;
  };
  float h[4];
  cudaMemsetAsync(acc, 0, sizeof(double) * 4, st);
  lap_apply_kernel<<<blocks, 256, 0, st>>>(L, d_x, ap, nullptr);
  cg_init_kernel<<<blocks, 256, 0, st>>>(n, d_rhs, ap, r, p, acc);
  cg_store_rr_kernel<<<1, 1, 0, st>>>(acc, scal, 0);
  cudaMemcpyAsync(h, scal, sizeof(float), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess || !check()) goto done;
  {
    const float rr_init = h[0];
    if (std::sqrt(rr_init) < abs_tol) goto done;
    for (int it = 0; it < max_iters; ++it) {
      iters = it + 1;
      cudaMemsetAsync(acc, 0, sizeof(double) * 2, st);
      lap_apply_kernel<<<blocks, 256, 0, st>>>(L, p, ap, acc);
      cg_alpha_kernel<<<1, 1, 0, st>>>(acc, scal);
      cg_update_kernel<<<blocks, 256, 0, st>>>(n, scal, p, ap, d_x, r, acc + 1);
      cg_store_rr_kernel<<<1, 1, 0, st>>>(acc + 1, scal, 2);
      cudaMemcpyAsync(h, scal, sizeof(float) * 3, cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess || !check()) goto done;
      const float rr = h[2];
      if (std::sqrt(rr / rr_init) < rel_tol) break;
      cg_direction_kernel<<<blocks, 256, 0, st>>>(n, scal, r, p, mode);
      cg_shift_rr_kernel<<<1, 1, 0, st>>>(scal);
      if (!check()) goto done;
    }
  }
done:
  cudaStreamSynchronize(st);
  cudaFree(buf);
  cudaFree(acc);
  cudaFree(scal);
  if (h_iters) *h_iters = iters;
  return status;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of wap_cg_screened_laplacian.
//
// Some callers cannot let a library allocate device memory on their behalf:
// an application whose memory pool has already reserved the device (an extra
// cudaMalloc then fails with out-of-memory), or a serving loop that keeps
// other streams busy and cannot absorb the device-wide synchronisation that
// cudaFree implies.  This entry point keeps its work vectors (r, p, Ap), its
// FP64 dot-product accumulators and its scalars in one fixed array below,
// which every GPU that loads the library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace wap {
namespace {

constexpr size_t kNoAllocVecBytes = sizeof(float) * 3 * (size_t)WAP_CG_NOALLOC_MAX_VOXELS;
constexpr size_t kNoAllocBytes = kNoAllocVecBytes + 256;  // + 4 doubles, 4 floats, padding

// The scratch every call shares: r, p, Ap, then the accumulators and scalars.
static __device__ __align__(256) unsigned char g_cg_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch, looked up once per device (host code cannot
// use the symbol itself: on the host it names a stand-in, not device memory).
std::mutex g_noalloc_mu;
void *g_noalloc_addr[128] = {nullptr};

int noalloc_scratch(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return WAP_ENODEV;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_cg_noalloc_scratch) != cudaSuccess || !p) return WAP_ECUDA;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return WAP_OK;
}

}  // namespace
}  // namespace wap

extern "C" int wap_cg_screened_laplacian_noalloc(void *cuda_stream, const int *dims, float a, float b,
                                                 const float *d_rhs, float *d_x, float rel_tol, int max_iters,
                                                 float abs_tol, int mode, int *h_iters) {
  if (!dims || !d_rhs || !d_x || dims[0] < 1 || dims[1] < 1 || dims[2] < 1 || max_iters < 0) return WAP_EINVAL;
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  if (n > (size_t)WAP_CG_NOALLOC_MAX_VOXELS) return WAP_ETOOBIG;
  void *base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc != WAP_OK) return rc;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  unsigned char *bytes = (unsigned char *)base;
  float *r = (float *)bytes, *p = r + n, *ap = r + 2 * n;
  double *acc = (double *)(bytes + kNoAllocVecBytes);
  float *scal = (float *)(bytes + kNoAllocVecBytes + 4 * sizeof(double));
  const Lap L{dims[0], dims[1], dims[2], a, b};
  const unsigned blocks = (unsigned)((n + 255) / 256);
  int iters = 0;
  float h[4];
  // The accumulators keep the previous call's sums: clear them before use.
  if (cudaMemsetAsync(acc, 0, sizeof(double) * 4, st) != cudaSuccess) return WAP_ECUDA;
  lap_apply_kernel<<<blocks, 256, 0, st>>>(L, d_x, ap, nullptr);
  cg_init_kernel<<<blocks, 256, 0, st>>>(n, d_rhs, ap, r, p, acc);
  cg_store_rr_kernel<<<1, 1, 0, st>>>(acc, scal, 0);
  if (cudaMemcpyAsync(h, scal, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return WAP_ECUDA;
  const float rr_init = h[0];
  if (!(std::sqrt(rr_init) < abs_tol)) {
    for (int it = 0; it < max_iters; ++it) {
      iters = it + 1;
      cudaMemsetAsync(acc, 0, sizeof(double) * 2, st);
      lap_apply_kernel<<<blocks, 256, 0, st>>>(L, p, ap, acc);
      cg_alpha_kernel<<<1, 1, 0, st>>>(acc, scal);
      cg_update_kernel<<<blocks, 256, 0, st>>>(n, scal, p, ap, d_x, r, acc + 1);
      cg_store_rr_kernel<<<1, 1, 0, st>>>(acc + 1, scal, 2);
      if (cudaMemcpyAsync(h, scal, sizeof(float) * 3, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return WAP_ECUDA;
      if (std::sqrt(h[2] / rr_init) < rel_tol) break;
      cg_direction_kernel<<<blocks, 256, 0, st>>>(n, scal, r, p, mode);
      cg_shift_rr_kernel<<<1, 1, 0, st>>>(scal);
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return WAP_ECUDA;
  if (h_iters) *h_iters = iters;
  return WAP_OK;
}
