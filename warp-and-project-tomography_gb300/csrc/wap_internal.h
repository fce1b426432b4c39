// Shared device/host definitions of the GB300 warp-and-project library.
//
// Every translation unit is compiled with -fmad=false: the reference defines
// its numbers without fused multiply-add, and the parity contract (sample
// counts and traversal bit-exact, projections and volumes reproducible)
// depends on each float operation rounding where the reference's does.
// Kernels that are allowed to differ use explicit __fmaf_rn.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

struct wap_ctx;

namespace wap {

// The stream a context orders its work on (capi.cpp).
cudaStream_t ctx_stream(wap_ctx *ctx);

// Per-projection geometry, produced on the host by geometry.cpp
// (TypicalRayProducer.cpp:157-232) and read by the projector kernels.
struct ProjGeom {
  float p2m[16];    // pixels -> model (inverse of V2P * Proj * MV)
  float m2v[16];    // model -> voxel
  float mvv2m[16];  // MV * V2M: voxel -> camera, used by the voxel-driven BP
  float eye[4];     // source position in model space
};

struct ScanDesc;  // forward (wap.h's wap_scan_desc is layout-compatible)

// The reference's min/max macros: ((a) < (b)) ? (a) : (b)
// (RayCaster.core.h:22-28, WaP_Tomo.cpp:170-176).
__host__ __device__ __forceinline__ float mac_min(float a, float b) { return (a < b) ? a : b; }
__host__ __device__ __forceinline__ float mac_max(float a, float b) { return (a > b) ? a : b; }
__host__ __device__ __forceinline__ int mac_mini(int a, int b) { return (a < b) ? a : b; }
__host__ __device__ __forceinline__ int mac_maxi(int a, int b) { return (a > b) ? a : b; }
// std::min / std::max argument order (advection.h, optical_flow.h).
__host__ __device__ __forceinline__ float std_min(float a, float b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ float std_max(float a, float b) { return (a < b) ? b : a; }

// Column-major 4x4 times vector, summed left to right (Matrix4x4.h).
__host__ __device__ __forceinline__ void mat4_vec(const float *M, float x, float y, float z, float w, float out[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) out[r] = M[r] * x + M[4 + r] * y + M[8 + r] * z + M[12 + r] * w;
}

// ---------------------------------------------------------------------------
// Job descriptors: one kernel launch serves many independent frames.
// ---------------------------------------------------------------------------
struct FpJob {
  const float *vol;   // volume to project
  int proj;           // projection index (geometry row, measured row)
  float *img;         // optional: projection (W*H)
  float *len;         // optional: ray length
  float *weight;      // optional: sample count
  const float *meas;  // optional: measured projection -> fused correction
  float *dual;        // optional: PSART dual row (y = 0 when null)
  float *corr;        // correction output when meas != null
};

struct BpJob {
  float *vol;         // SART: volume updated in place; delta mode: accumulator
  const float *corr;  // correction image (W*H)
  int proj;           // geometry row
  int box[6];         // x0,x1,y0,y1,z0,z1 (half-open)
};

struct SplatJob {
  const float *corr;
  int proj;
  float *contrib;
  float *weight;
};

// Launch helpers (implemented in the .cu files).
// bricked: the jobs' volumes are in the 4x4x4 brick layout (launch_brick).
// half (the precision form): the brick copies are FP16 and each ray's sum is
// Kahan-compensated FP32; sample counts and ray lengths are unchanged.
cudaError_t launch_forward(const ProjGeom *d_geom, const FpJob *d_jobs, int njobs, const int dims[3], int W, int H,
                           float sd, double alpha, cudaStream_t st, bool bricked = false, bool half = false);
// Floats of a volume's brick layout (dims rounded up to multiples of 4), and
// the conversion of a linear volume into it.
size_t brick_floats(const int dims[3]);
cudaError_t launch_brick(const float *vol, float *out, const int dims[3], cudaStream_t st);
// The volumes of njobs projection jobs (d_jobs[j].vol) into slots j of out
// (brick_floats(dims) floats apart), one launch (njobs <= 65535).
cudaError_t launch_brick_jobs(const FpJob *d_jobs, int njobs, float *out, const int dims[3], cudaStream_t st,
                              bool half = false);
cudaError_t launch_bp_voxel(const ProjGeom *d_geom, const BpJob *d_jobs, int njobs, int maxbox[3], const int dims[3],
                            int W, int H, double halfW, double halfH, float sdd, double ds, double alpha, float gmax,
                            int mode, int exact, cudaStream_t st);
// direct: every tap a global atomic (the plain form); otherwise the
// shared-memory slab accumulation of bp_ray_kernel.
cudaError_t launch_ray_splat(const ProjGeom *d_geom, const SplatJob *d_jobs, int njobs, const int dims[3], int W,
                             int H, float sd, cudaStream_t st, bool direct = false);
// ---------------------------------------------------------------------------
// Work-queue forms for a batch of scans of different sizes: one persistent
// launch covers every job of a step; its blocks take work items (a pixel
// tile, a voxel block, a brick tile of one job) from a counter that the
// launcher zeroes first.  Jobs are listed in item order (item0 ascending).
// ---------------------------------------------------------------------------
struct QFpJob {
  FpJob job;
  const ProjGeom *geom;
  int n[3], W, H;
  float sd;
  double alpha;
  int bricked;  // 1: job.vol is a brick-layout copy; 2: an FP16 one (the precision form)
  int tiles_x;  // pixel tiles across the detector (set for the launcher's tile shape)
  int item0;
};
struct QBpParams {  // BpParams (projector.cu) as the host fills it
  int nx, ny, W, H;
  double halfW, halfH;
  float sdd;
  double ds;
  int float_ok;
  double alpha;
  float gmax, halfWf, halfHf, dsf, alphaf, alphal, wlim, hlim;
};
struct QBpJob {
  BpJob job;
  const ProjGeom *geom;
  QBpParams P;
  int bx, by;  // voxel blocks across the box in x and y (the launcher's block shape)
  int item0;
};
struct QBrickJob {
  const float *vol;  // linear volume
  float *out;        // its brick-layout copy
  int n[3];
  int half;          // the copy in FP16 (the precision form)
  int tx, ty;        // 32x4x4 tiles across x and y
  int item0;
};
QBpParams make_bp_params(const int dims[3], int W, int H, double halfW, double halfH, float sdd, double ds,
                         double alpha, float gmax);
// Tile shapes: fp 0 = 16x8 pixels (128 threads), 1 = 8x8 (64), 2 = 32x8 (256);
// bp 0 = 32x4x2 voxels, 1 = 32x8x1, 2 = 32x2x4 (256 threads).
constexpr int kFpShapes = 3, kBpShapes = 3;
void fp_shape_tile(int shape, int &tw, int &th);
void bp_shape_block(int shape, int &bx, int &by, int &bz);
// Fill each job's per-shape tile counts and first item in host copies (the
// caller uploads them); return the launch's item count.
int fp_queue_items(QFpJob *h_jobs, int njobs, int shape);
int bp_queue_items(QBpJob *h_jobs, int njobs, int shape);
int brick_queue_items(QBrickJob *h_jobs, int njobs);
cudaError_t launch_fp_queue(const QFpJob *d_jobs, int njobs, int total, int *d_counter, int shape, cudaStream_t st);
cudaError_t launch_bp_queue(const QBpJob *d_jobs, int njobs, int total, int *d_counter, int shape, int exact,
                            int mode, cudaStream_t st);
cudaError_t launch_brick_queue(const QBrickJob *d_jobs, int njobs, int total, int *d_counter, cudaStream_t st);
// Asks every work-queue kernel's occupancy now (before a stream capture).
void warm_queue_kernels();

// The ray-driven SART update over a job's box: where weight > 0,
// vol = clamp(vol + alpha * (contrib / weight), 0, gmax) in float.
struct RayUpdJob {
  float *vol;
  const float *contrib;
  const float *weight;
  int box[6];
};
cudaError_t launch_ray_update(const RayUpdJob *d_jobs, int njobs, const int maxbox[3], const int dims[3],
                              double alpha, float gmax, cudaStream_t st);
cudaError_t launch_correction(int n, const float *meas, const float *img, const float *len, float *dual,
                              double alpha, float *corr, cudaStream_t st);

struct AdvectJob {
  const float *vel;  // 3 planar channels
  const float *src;  // nc planar channels
  float *out;        // nc planar channels
  float dt;
};
// Cell-centre world coordinates per axis (advection.h:24-29), sum(dims) floats.
void world_table(const int dims[3], const float aabb[6], float *h);
// fast: the precision form's fused-multiply-add cubic (results within a
// tolerance); false: the reference's arithmetic, bit for bit.
// d_flags (njobs ints of scratch, may be NULL): with it, each job's velocity
// is range-checked first and cell-centre samples take their centre tap (same
// bits); without it every sample is the full clamped tricubic.
cudaError_t launch_advect(const int dims[3], const float aabb[6], const float *d_world, const AdvectJob *d_jobs,
                          int njobs, int nc, cudaStream_t st, bool fast = false, int *d_flags = nullptr);
// vol = clamp_cut(vol + alpha*adv) then max(vol*roi, 0) (WaP_Tomo.cpp:1378-1412);
// floor = false leaves out the max(., 0).
cudaError_t launch_wap_accumulate(size_t n, float *vol, const float *adv, double alpha, float gmax, cudaStream_t st,
                                  bool floor = true);
cudaError_t launch_roi_floor(size_t n, float *vol, cudaStream_t st);
// Adds to *d_bad the number of n pseudo-random inputs (from seed) on which the
// warp's packed-pair cubic and its scalar cubic differ in bits, in both the
// reference and the fast arithmetic.
cudaError_t launch_cubic_pair_check(unsigned long long n, unsigned long long seed, unsigned long long *d_bad,
                                    cudaStream_t st);
struct AccJob {
  float *vol;
  const float *adv;
};
cudaError_t launch_wap_accumulate_batch(const AccJob *d_jobs, int njobs, size_t n, double alpha, float gmax,
                                        cudaStream_t st);
cudaError_t launch_max_reduce(const float *d, size_t n, unsigned *d_bits, cudaStream_t st);
float decode_max_bits(unsigned b);

// Device bytes the precision form adds to a job (wap_job_device_bytes counts
// the FP32 path): the flow solver's FP16 pair state, 64 bytes per voxel of
// every pyramid level (capi.cpp).
size_t flow_pairs_bytes(const int vol[3], int flow_scales, float flow_eta);

}  // namespace wap
