// Conjugate gradients on a volume (image_cg::cg, cg.h:11-55, with the
// image_blas vector operations of image_blas.h:9-91).  cg.h has no caller in
// the reference; the operator here is the SPD screened Laplacian
// A x = a x - b (sum of the 6 clamped neighbours - 6 x), the system the
// reference's test-free CG would be pointed at.  Vectors are FP32; every dot
// product is a warp-shuffle reduction accumulated in FP64, and the scalar
// recurrences (alpha, beta, the convergence ratio) stay on the device.
//
// The dot products are deterministic: each block writes its FP64 partial sum
// to its own slot, and one block adds the slots in a fixed order.  A solve
// therefore gives the same bits and the same iteration count on every run,
// which the allocating and the allocation-free entry points below share.
#include <cmath>

#include "c_boundary.h"
#include "wap/wap.h"
#include "wap_internal.h"

namespace wap {
namespace {

constexpr int kThreads = 256;

// Sum of v over the block in a fixed order; valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int tid = threadIdx.x;
  if ((tid & 31) == 0) sh[tid >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (tid == 0)
    for (int w = 0; w < kThreads / 32; ++w) s += sh[w];
  return s;
}

// The block's partial sum into part[blockIdx.x] (part may be null).
__device__ __forceinline__ void block_partial(double v, double *part) {
  if (!part) return;
  const double s = block_sum(v);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// One block of kThreads: sum of part[0..nb) in a fixed order; valid in thread 0.
__device__ __forceinline__ double sum_partials(const double *__restrict__ part, int nb) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += kThreads) v += part[i];
  return block_sum(v);
}

struct Lap {
  int nx, ny, nz;
  float a, b;
};

// out = A in; part[block] = this block's share of dot(in, out)
__global__ void lap_apply_kernel(Lap L, const float *__restrict__ in, float *__restrict__ out, double *part) {
  const size_t n = (size_t)L.nx * L.ny * L.nz;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < n) {
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((size_t)L.nx * L.ny));
    const size_t sy = L.nx, sz = (size_t)L.nx * L.ny;
    const float xc = in[t];
    const float s = in[i > 0 ? t - 1 : t] + in[i < L.nx - 1 ? t + 1 : t] + in[j > 0 ? t - sy : t] +
                    in[j < L.ny - 1 ? t + sy : t] + in[k > 0 ? t - sz : t] + in[k < L.nz - 1 ? t + sz : t];
    const float y = L.a * xc - L.b * (s - 6.0f * xc);
    out[t] = y;
    v = (double)xc * (double)y;
  }
  block_partial(v, part);
}

// r = b - Ap, p = r, part[block] = share of dot(r, r)
__global__ void cg_init_kernel(size_t n, const float *__restrict__ rhs, const float *__restrict__ ap,
                               float *__restrict__ r, float *__restrict__ p, double *part) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < n) {
    const float rv = (float)((double)rhs[t] + (double)ap[t] * -1.0);
    r[t] = rv;
    p[t] = rv;
    v = (double)rv * (double)rv;
  }
  block_partial(v, part);
}

// scal[0] = rr_old, scal[1] = alpha = rr_old / pAp (pAp from the partials).
__global__ void cg_alpha_kernel(const double *__restrict__ part, int nb, float *__restrict__ scal) {
  const double pap = sum_partials(part, nb);
  if (threadIdx.x == 0) scal[1] = scal[0] / (float)pap;
}

// x += alpha p; r += (-alpha) Ap; part[block] = share of dot(r, r)
__global__ void cg_update_kernel(size_t n, const float *__restrict__ scal, const float *__restrict__ p,
                                 const float *__restrict__ ap, float *__restrict__ x, float *__restrict__ r,
                                 double *part) {
  const float alpha = scal[1];
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < n) {
    x[t] = x[t] + p[t] * alpha;
    const float rv = r[t] + ap[t] * -alpha;
    r[t] = rv;
    v = (double)rv * (double)rv;
  }
  block_partial(v, part);
}

// p = r + beta p (mode 0) or p = r + 0 * beta (mode 1, the reference's aliasing).
__global__ void cg_direction_kernel(size_t n, const float *__restrict__ scal, const float *__restrict__ r,
                                    float *__restrict__ p, int mode) {
  const float beta = scal[2] / scal[0];
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  p[t] = mode == 1 ? r[t] + 0.0f * beta : r[t] + p[t] * beta;
}

// scal[slot] = (float) sum of the partials
__global__ void cg_store_rr_kernel(const double *__restrict__ part, int nb, float *__restrict__ scal, int slot) {
  const double s = sum_partials(part, nb);
  if (threadIdx.x == 0) scal[slot] = (float)s;
}

__global__ void cg_shift_rr_kernel(float *__restrict__ scal) { scal[0] = scal[2]; }

// Device buffers of one solve: r, p, Ap (n floats each), two partial-sum
// arrays (nb doubles each) and four scalars.
struct CgBufs {
  float *r, *p, *ap;
  double *part_pap, *part_rr;
  float *scal;
};

// The solve itself, shared by both entry points.  Errors from the caller's
// earlier work are left pending and reported as WAP_ECUDA before anything is
// launched; errors of this solve's own launches are consumed.  *h_iters is
// written on every path.
int cg_solve(cudaStream_t st, const int *dims, float a, float b, const float *d_rhs, float *d_x, float rel_tol,
             int max_iters, float abs_tol, int mode, const CgBufs &B, int *h_iters) {
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  const Lap L{dims[0], dims[1], dims[2], a, b};
  const int nb = (int)((n + kThreads - 1) / kThreads);
  int iters = 0, status = WAP_OK;
  float h[4];
  auto failed = [&](cudaError_t e) {
    const cudaError_t pending = cudaGetLastError();  // this solve's own launch errors
    if (e != cudaSuccess || pending != cudaSuccess) status = WAP_ECUDA;
    return status != WAP_OK;
  };
  if (cudaPeekAtLastError() != cudaSuccess) {
    status = WAP_ECUDA;
    goto done;
  }
  lap_apply_kernel<<<nb, kThreads, 0, st>>>(L, d_x, B.ap, nullptr);
  cg_init_kernel<<<nb, kThreads, 0, st>>>(n, d_rhs, B.ap, B.r, B.p, B.part_rr);
  cg_store_rr_kernel<<<1, kThreads, 0, st>>>(B.part_rr, nb, B.scal, 0);
  if (failed(cudaMemcpyAsync(h, B.scal, sizeof(float), cudaMemcpyDeviceToHost, st)) ||
      failed(cudaStreamSynchronize(st)))
    goto done;
  {
    const float rr_init = h[0];
    if (std::sqrt(rr_init) < abs_tol) goto done;
    for (int it = 0; it < max_iters; ++it) {
      iters = it + 1;
      lap_apply_kernel<<<nb, kThreads, 0, st>>>(L, B.p, B.ap, B.part_pap);
      cg_alpha_kernel<<<1, kThreads, 0, st>>>(B.part_pap, nb, B.scal);
      cg_update_kernel<<<nb, kThreads, 0, st>>>(n, B.scal, B.p, B.ap, d_x, B.r, B.part_rr);
      cg_store_rr_kernel<<<1, kThreads, 0, st>>>(B.part_rr, nb, B.scal, 2);
      if (failed(cudaMemcpyAsync(h, B.scal, sizeof(float) * 3, cudaMemcpyDeviceToHost, st)) ||
          failed(cudaStreamSynchronize(st)))
        goto done;
      if (std::sqrt(h[2] / rr_init) < rel_tol) break;
      cg_direction_kernel<<<nb, kThreads, 0, st>>>(n, B.scal, B.r, B.p, mode);
      cg_shift_rr_kernel<<<1, 1, 0, st>>>(B.scal);
      if (failed(cudaSuccess)) goto done;
    }
  }
done:
  if (status == WAP_OK && failed(cudaStreamSynchronize(st))) status = WAP_ECUDA;
  if (h_iters) *h_iters = iters;
  return status;
}

bool cg_args_ok(const int *dims, const float *d_rhs, const float *d_x, int max_iters) {
  return dims && d_rhs && d_x && dims[0] >= 1 && dims[1] >= 1 && dims[2] >= 1 && max_iters >= 0;
}

}  // namespace
}  // namespace wap

using namespace wap;

extern "C" int wap_cg_screened_laplacian(wap_ctx *ctx, const int *dims, float a, float b, const float *d_rhs,
                                         float *d_x, float rel_tol, int max_iters, float abs_tol, int mode,
                                         int *h_iters) try {
  if (!ctx || !cg_args_ok(dims, d_rhs, d_x, max_iters)) return WAP_EINVAL;
  cudaStream_t st = ctx_stream(ctx);
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  const size_t nb = (n + kThreads - 1) / kThreads;
  float *buf = nullptr, *scal = nullptr;
  double *part = nullptr;
  if (cudaMalloc(&buf, sizeof(float) * 3 * n) != cudaSuccess || cudaMalloc(&part, sizeof(double) * 2 * nb) != cudaSuccess ||
      cudaMalloc(&scal, sizeof(float) * 4) != cudaSuccess) {
    cudaGetLastError();  // the failed allocation's error is reported as WAP_ENOMEM
    cudaFree(buf);
    cudaFree(part);
    if (h_iters) *h_iters = 0;
    return WAP_ENOMEM;
  }
  const CgBufs B{buf, buf + n, buf + 2 * n, part, part + nb, scal};
  const int status = cg_solve(st, dims, a, b, d_rhs, d_x, rel_tol, max_iters, abs_tol, mode, B, h_iters);
  cudaFree(buf);
  cudaFree(part);
  cudaFree(scal);
  return status;
} WAP_CATCH

// ---------------------------------------------------------------------------
// Allocation-free variant of wap_cg_screened_laplacian.
//
// Some callers cannot let a library allocate device memory on their behalf:
// an application whose memory pool has already reserved the device (an extra
// cudaMalloc then fails with out-of-memory), or a serving loop that keeps
// other streams busy and cannot absorb the device-wide synchronisation that
// cudaFree implies.  This entry point keeps its work vectors (r, p, Ap), its
// FP64 partial sums and its scalars in one fixed array below, which every GPU
// that loads the library holds until the process exits.  It runs the same
// kernels in the same order as the allocating entry point, so both give the
// same bits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace wap {
namespace {

constexpr size_t kNoAllocVecBytes = sizeof(float) * 3 * (size_t)WAP_CG_NOALLOC_MAX_VOXELS;
constexpr size_t kNoAllocBlocks = ((size_t)WAP_CG_NOALLOC_MAX_VOXELS + kThreads - 1) / kThreads;
constexpr size_t kNoAllocPartBytes = sizeof(double) * 2 * kNoAllocBlocks;
constexpr size_t kNoAllocBytes = kNoAllocVecBytes + kNoAllocPartBytes + 256;  // + 4 scalars, padding

// The scratch every call shares: r, p, Ap, the two partial-sum arrays, the scalars.
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
                                                 float abs_tol, int mode, int *h_iters) try {
  if (h_iters) *h_iters = 0;
  if (!cg_args_ok(dims, d_rhs, d_x, max_iters)) return WAP_EINVAL;
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  if (n > (size_t)WAP_CG_NOALLOC_MAX_VOXELS) return WAP_ETOOBIG;
  void *base = nullptr;
  const int rc = noalloc_scratch(&base);
  if (rc != WAP_OK) return rc;
  unsigned char *bytes = (unsigned char *)base;
  float *r = (float *)bytes;
  double *part = (double *)(bytes + kNoAllocVecBytes);
  float *scal = (float *)(bytes + kNoAllocVecBytes + kNoAllocPartBytes);
  // Every slot the solve reads is written by the same solve before it is
  // read (partials by the block that owns them, scalars by the reduction
  // kernels), so nothing left by the previous call needs clearing.
  const CgBufs B{r, r + n, r + 2 * n, part, part + kNoAllocBlocks, scal};
  return cg_solve((cudaStream_t)cuda_stream, dims, a, b, d_rhs, d_x, rel_tol, max_iters, abs_tol, mode, B, h_iters);
} WAP_CATCH
