// C ABI (include/wap/wap.h) of the GB300 warp-and-project library: the
// context, its device arenas, and the host-side orchestration of PSART's
// loops (WaP_Tomo.cpp:473-1678) and the flow solver's control flow
// (optical_flow.h:409-828, 1002-1126) around the kernels.
//
// Device layout: the level's F frame volumes are one contiguous arena
// (frame-major, CImg order inside a frame), likewise the flows (3 planar
// channels per frame) and the CP state.  Independent frames are batched into
// single launches (job tables), so a 64^3 frame set fills the GPU the way one
// 256^3 frame does.  Nothing here falls back to the CPU: every numeric step
// is a kernel in this library, and a missing GPU is an error.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "c_boundary.h"
#include "wap/wap.h"
#include "wap/wap_serve.h"
#include "wap_flow.h"
#include "wap_geometry.h"
#include "wap_internal.h"

using namespace wap;

namespace {

// Device blocks of destroyed contexts, kept for the next context instead of
// cudaFree, which synchronises the whole device (and so would stall every
// other reconstruction of a request loop each time one finishes).  Only
// wap_destroy recycles, after the context's stream has drained; keyed by
// (device, capacity); a request takes the smallest block that fits with at
// most 1/8 (or 2 MiB) slack.  An allocation that fails empties the cache of
// that device and retries.
std::mutex g_cache_mu;
std::multimap<std::pair<int, size_t>, void *> g_cache;
size_t g_cache_bytes = 0;
thread_local bool g_recycle = false;

void *cache_take(size_t b, size_t &cap) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_cache_mu);
  auto it = g_cache.lower_bound(std::make_pair(dev, b));
  // blocks of 1 MiB or more may come from a cached block up to 1/8 larger;
  // smaller requests take only a block of their own size
  const size_t slack = b >= ((size_t)1 << 20) ? b / 8 : 0;
  if (it == g_cache.end() || it->first.first != dev || it->first.second > b + slack) return nullptr;
  cap = it->first.second;
  void *p = it->second;
  g_cache.erase(it);
  g_cache_bytes -= cap;
  return p;
}

void cache_put(void *p, size_t cap) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaFree(p);
    return;
  }
  std::lock_guard<std::mutex> lk(g_cache_mu);
  g_cache.emplace(std::make_pair(dev, cap), p);
  g_cache_bytes += cap;
}

size_t cache_trim(int dev) {  // dev < 0: every device
  std::lock_guard<std::mutex> lk(g_cache_mu);
  size_t freed = 0;
  for (auto it = g_cache.begin(); it != g_cache.end();) {
    if (dev >= 0 && it->first.first != dev) {
      ++it;
      continue;
    }
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(it->first.first);
    cudaFree(it->second);
    cudaSetDevice(cur);
    freed += it->first.second;
    g_cache_bytes -= it->first.second;
    it = g_cache.erase(it);
  }
  return freed;
}

// CUDA events owned by one call, destroyed on every return path.
struct ScopedEvents {
  std::vector<cudaEvent_t> e;
  explicit ScopedEvents(size_t n) : e(n, nullptr) {}
  ScopedEvents(const ScopedEvents &) = delete;
  ScopedEvents &operator=(const ScopedEvents &) = delete;
  ~ScopedEvents() {
    for (cudaEvent_t x : e)
      if (x) cudaEventDestroy(x);
  }
  cudaError_t create() {
    for (auto &x : e) {
      const cudaError_t r = cudaEventCreate(&x);
      if (r != cudaSuccess) {
        x = nullptr;
        return r;
      }
    }
    return cudaSuccess;
  }
  cudaEvent_t operator[](size_t i) const { return e[i]; }
};

struct DevMem {
  void *p = nullptr;
  size_t bytes = 0;  // capacity
  size_t want = 0;   // the largest size asked of this block since it was (re)allocated
  DevMem() = default;
  DevMem(const DevMem &) = delete;
  DevMem &operator=(const DevMem &) = delete;
  ~DevMem() {
    if (p && g_recycle) cache_put(p, bytes);
    else release();
  }
  void release() {  // in-flight work may still use the block: a synchronising free
    if (p) cudaFree(p);
    p = nullptr;
    bytes = want = 0;
  }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) {
      want = std::max(want, b);
      return cudaSuccess;
    }
    release();
    const size_t ask = b ? b : 16;
    size_t cap = 0;
    if ((p = cache_take(ask, cap)) != nullptr) {
      bytes = cap;
      want = ask;
      return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(&p, ask);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      int dev = 0;
      cudaGetDevice(&dev);
      if (cache_trim(dev) > 0) e = cudaMalloc(&p, ask);
    }
    if (e == cudaSuccess) bytes = want = ask;
    else p = nullptr;
    return e;
  }
  template <class T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
};

struct Status {
  int code;
};

// Exhaustive proofs of the fast division paths, per (device, key).
std::mutex g_proof_mutex;
std::map<std::pair<int, uint64_t>, int> g_proofs;
// Autotuned primal-dual plans shared by every context of the process, so a
// request loop's jobs tune each grid size once: (device, nx, ny, nz, FP16
// storage, TMA form available) -> (form, z-chunk).
std::mutex g_plan_mutex;
std::map<std::tuple<int, int, int, int, int, int>, std::pair<int, int>> g_plans;

// Flow-solver workspace for one grid size (reused across pairs and calls).
struct FlowWork {
  int n[3] = {0, 0, 0};
  DevMem va, vb, y, y2, u, kty, kx4prev, warp, acc, err, world, tma_err;
  float aabb_key[6] = {0, 0, 0, 0, 0, 0};
  // Tensor maps of the TMA-fed form: y over (y, y2), v over (va, vb), u.
  int tma_state = 0;  // 0: not made, 1: made, -1: unavailable for this grid
  PdTmaMap ymap[2], vmap[2], umap;
  // The precision form's FP16 copies of y, v, u and their tensor maps.
  int h_state = 0;
  DevMem yh[2], vh[2], uh;
  PdTmaMap hymap[2], hvmap[2], humap;
};

// Multiscale pyramid buffers for one finest size.
struct PyramidLevel {
  int d[3];
  DevMem i1, i2, v, y;
};

}  // namespace

struct wap_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  wap_scan_desc scan{};
  ScanGeometry sg{};
  std::vector<double> angles;
  std::vector<ProjGeom> h_geom;
  DevMem geom;
  float sd = 0.0f;
  double halfW = 0.0, halfH = 0.0;
  float gmax = 0.0f;
  DevMem projs_own;
  const float *projs = nullptr;
  size_t np = 0, nv = 0;

  // time level
  int level = -1, F = 0;
  std::vector<int> st, en;
  std::vector<float> ft;
  float tunit = 0.0f;
  DevMem vols, flows, ytv, ytp, xbar, xprev, zero_vol;
  DevMem dual, corr, warped, delta, back;
  int maxwin = 0;

  // job tables and scratch
  DevMem jobs_fp, jobs_bp, jobs_adv, jobs_acc, jobs_misc;
  DevMem world;  // cell-centre table of the scan grid
  DevMem maxbits;
  std::map<std::tuple<int, int, int>, std::unique_ptr<FlowWork>> flow_work;
  std::vector<std::unique_ptr<PyramidLevel>> pyramid;
  DevMem blur_a, blur_b, rs_a, rs_b;
  DevMem pyr_b1, pyr_b2;  // blurred full-size flow inputs
  DevMem adv_tab;         // cell-centre table of a wap_advect call
  DevMem adv_flags;       // per advect job: its velocity's range check
  DevMem bricks;          // brick-layout copies of the volumes a projection batch reads
  DevMem jobs_fpb;        // the batch's projection jobs pointing at those copies
  int fp_bricks = 1;      // 1: the forward projector reads brick-layout copies (same bits, faster)
  int bp_ray = 0;         // 1: SART backprojects ray-driven, normalised by the column sums
  int splat_direct = 0;   // 1: the ray-driven splat issues a global atomic per tap (comparison form)
  DevMem ray_acc;         // contributions and weights of a ray-driven SART step (2 V per frame job)
  DevMem jobs_splat, jobs_rupd;
  std::map<std::pair<int, int>, std::unique_ptr<DevMem[]>> resize_tables;
  DevMem cg_buf;

  wap_stats stats{};
  int profiling = 0;
  int pd_form = 0;    // 0: autotuned, 1: fused kernel, 2: primal + dual kernels
  int pd_zchunk = 0;  // 0: autotuned / default
  int flow_bits = 32; // 16: the flow solver's y, v, u stored in FP16 (the precision form)
  // flow pairs of an outer iteration run concurrently on this many lanes (1: in
  // turn; 0: automatic, kAutoLanesSmall for a flow grid of at most
  // kAutoLanesSmallVoxels, whose levels are latency-bound, else 2)
  int flow_lanes = 0;
  std::vector<wap_ctx *> lanes;  // the lanes: helper compute contexts, each with its own stream and workspaces
  std::set<std::tuple<int, int, int, int, int, int>> lanes_tuned;  // flow shapes whose plans are tuned
  std::map<std::tuple<int, int, int>, std::pair<int, int>> pd_plans;  // grid -> (form, zchunk)
  std::map<std::tuple<int, int, int>, std::pair<int, int>> pd_plans16;  // the same for FP16 storage
  wap_observer_fn observer = nullptr;
  void *observer_user = nullptr;
  std::vector<cudaEvent_t> pd_events;  // pairs, reused per 50-iteration chunk
  std::string err;
};

namespace wap {
cudaStream_t ctx_stream(wap_ctx *ctx) { return ctx->stream; }
}  // namespace wap

namespace {

int fail(wap_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CU(expr)                                                                                     \
  do {                                                                                               \
    cudaError_t _e = (expr);                                                                         \
    if (_e != cudaSuccess) return fail(ctx, WAP_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

#define KL(expr)          \
  do {                    \
    CU(expr);             \
    ++ctx->stats.kernel_launches; \
  } while (0)

#define CHECK(cond, code, msg)                \
  do {                                        \
    if (!(cond)) return fail(ctx, code, msg); \
  } while (0)

#define TRY(expr)             \
  do {                        \
    int _r = (expr);          \
    if (_r != WAP_OK) return _r; \
  } while (0)

template <class T>
int upload(wap_ctx *ctx, DevMem &m, const std::vector<T> &h) {
  CU(m.ensure(sizeof(T) * h.size()));
  if (!h.empty()) CU(cudaMemcpyAsync(m.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
  return WAP_OK;
}

// Room for brick-layout copies of `floats` floats; without it (device memory
// exhausted) the projector reads the linear volumes, which gives the same bits.
bool brick_room(wap_ctx *ctx, size_t floats) {
  if (ctx->bricks.ensure(sizeof(float) * floats) == cudaSuccess) return true;
  cudaGetLastError();
  return false;
}

float *vol_ptr(wap_ctx *c, int f) { return c->vols.as<float>() + (size_t)f * c->nv; }
float *flow_ptr(wap_ctx *c, int f) { return c->flows.as<float>() + (size_t)f * 3 * c->nv; }

void sart_order(int pstart, int pend, std::vector<int> &order) {
  // front/back interleave of the window (WaP_Tomo.cpp:1449-1484).
  const int num = pend - pstart + 1;
  order.resize(num);
  for (int i = 0; i < num; ++i) order[i] = (i % 2 == 0) ? pstart + i / 2 : pend - i / 2;
}

// Reports an intermediate state to the observer once the stream has
// produced it.
int notify(wap_ctx *ctx, int event, int a, int b, const float *d) {
  if (!ctx->observer) return WAP_OK;
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->observer(ctx->observer_user, event, ctx->level, a, b, d);
  return WAP_OK;
}

bool has_scan(const wap_ctx *ctx) { return ctx->nv > 0 && !ctx->h_geom.empty(); }

int ensure_level_buffers(wap_ctx *ctx) {
  const size_t nv = ctx->nv, np = ctx->np, F = ctx->F;
  CU(ctx->corr.ensure(sizeof(float) * F * np));
  CU(ctx->dual.ensure(sizeof(float) * F * ctx->maxwin * np));
  CU(ctx->warped.ensure(sizeof(float) * F * nv));
  CU(ctx->delta.ensure(sizeof(float) * F * nv));
  CU(ctx->back.ensure(sizeof(float) * F * nv));
  return WAP_OK;
}

int roi_box(wap_ctx *ctx, int cut, int box[6]) {
  // m_roi = cut * dims / level-0 dims (WaP_Tomo.cpp:529-536).
  const int *d = ctx->scan.vol;
  for (int a = 0; a < 3; ++a) {
    const int r = (int)((float)cut * ((float)d[a] / (float)d[a]));
    box[2 * a] = r;
    box[2 * a + 1] = d[a] - r;
  }
  return WAP_OK;
}

// SART proximal operator on a set of frames at once (WaP_Tomo.cpp:1424-1678):
// frames step through their windows in lock-step; each step is one batched
// forward projection with the fused correction/dual epilogue and one batched
// backprojection.
int sart_frames(wap_ctx *ctx, const std::vector<int> &frames, int nb_sart, const int box[6], int exact) {
  const size_t np = ctx->np;
  const int W = ctx->scan.det[0], H = ctx->scan.det[1];
  CU(cudaMemsetAsync(ctx->dual.p, 0, sizeof(float) * ctx->F * ctx->maxwin * np, ctx->stream));
  std::vector<std::vector<int>> orders(frames.size());
  int maxnum = 0;
  for (size_t q = 0; q < frames.size(); ++q) {
    const int f = frames[q];
    sart_order(ctx->st[f], ctx->en[f], orders[q]);
    maxnum = std::max(maxnum, (int)orders[q].size());
  }
  std::vector<FpJob> fp;
  std::vector<BpJob> bp;
  std::vector<int> step_off(maxnum + 1, 0);
  for (int s = 0; s < maxnum; ++s) {
    step_off[s] = (int)fp.size();
    for (size_t q = 0; q < frames.size(); ++q) {
      if (s >= (int)orders[q].size()) continue;
      const int f = frames[q], pid = orders[q][s];
      FpJob j{};
      j.vol = vol_ptr(ctx, f);
      j.proj = pid;
      j.meas = ctx->projs;
      j.dual = ctx->dual.as<float>() + ((size_t)f * ctx->maxwin + (pid - ctx->st[f])) * np;
      j.corr = ctx->corr.as<float>() + (size_t)f * np;
      fp.push_back(j);
      BpJob b{};
      b.vol = vol_ptr(ctx, f);
      b.corr = j.corr;
      b.proj = pid;
      std::memcpy(b.box, box, sizeof(b.box));
      bp.push_back(b);
    }
  }
  step_off[maxnum] = (int)fp.size();
  // Brick layout: each step projects brick copies, made from the volumes the
  // previous step's backprojection just updated (jobs_fp keeps the linear
  // volumes for the conversion, jobs_fpb points at the copies).
  const size_t bf = brick_floats(ctx->scan.vol);
  int maxn = 0;
  for (int s = 0; s < maxnum; ++s) maxn = std::max(maxn, step_off[s + 1] - step_off[s]);
  const bool bricks = ctx->fp_bricks != 0 && brick_room(ctx, bf * maxn);
  if (bricks) {
    std::vector<FpJob> fpb = fp;
    for (int s = 0; s < maxnum; ++s)
      for (int q = step_off[s]; q < step_off[s + 1]; ++q) fpb[q].vol = ctx->bricks.as<float>() + (q - step_off[s]) * bf;
    TRY(upload(ctx, ctx->jobs_fpb, fpb));
  }
  TRY(upload(ctx, ctx->jobs_fp, fp));
  TRY(upload(ctx, ctx->jobs_bp, bp));
  int mb[3] = {box[1] - box[0], box[3] - box[2], box[5] - box[4]};
  // The precision form projects FP16 brick copies with compensated sums.
  const bool half = ctx->flow_bits == 16;
  // Ray-driven mode: each step's corrections are backprojected by the
  // matched ray-driven splat into per-job contribution / weight sums, and
  // the volume takes alpha * contribution / weight (SART's column-sum
  // normalisation) over the box.
  const bool ray = ctx->bp_ray != 0;
  if (ray) {
    CU(ctx->ray_acc.ensure(sizeof(float) * 2 * ctx->nv * (size_t)std::max(maxn, 1)));
    std::vector<SplatJob> sj;
    std::vector<RayUpdJob> uj;
    for (int s = 0; s < maxnum; ++s)
      for (int q = step_off[s]; q < step_off[s + 1]; ++q) {
        float *acc = ctx->ray_acc.as<float>() + (size_t)(q - step_off[s]) * 2 * ctx->nv;
        sj.push_back(SplatJob{fp[q].corr, fp[q].proj, acc, acc + ctx->nv});
        RayUpdJob u{};
        u.vol = bp[q].vol;
        u.contrib = acc;
        u.weight = acc + ctx->nv;
        std::memcpy(u.box, box, sizeof(u.box));
        uj.push_back(u);
      }
    TRY(upload(ctx, ctx->jobs_splat, sj));
    TRY(upload(ctx, ctx->jobs_rupd, uj));
  }
  for (int it = 1; it <= nb_sart; ++it)
    for (int s = 0; s < maxnum; ++s) {
      const int n = step_off[s + 1] - step_off[s];
      if (bricks)
        KL(launch_brick_jobs(ctx->jobs_fp.as<FpJob>() + step_off[s], n, ctx->bricks.as<float>(), ctx->scan.vol,
                             ctx->stream, half));
      KL(launch_forward(ctx->geom.as<ProjGeom>(), (bricks ? ctx->jobs_fpb : ctx->jobs_fp).as<FpJob>() + step_off[s],
                        n, ctx->scan.vol, W, H, ctx->sd, ctx->scan.alpha, ctx->stream, bricks, half && bricks));
      ctx->stats.fp_launches++;
      ctx->stats.projections += n;
      ctx->stats.backprojections += n;
      if (ray) {
        CU(cudaMemsetAsync(ctx->ray_acc.p, 0, sizeof(float) * 2 * ctx->nv * n, ctx->stream));
        KL(launch_ray_splat(ctx->geom.as<ProjGeom>(), ctx->jobs_splat.as<SplatJob>() + step_off[s], n, ctx->scan.vol,
                            W, H, ctx->sd, ctx->stream, ctx->splat_direct != 0));
        KL(launch_ray_update(ctx->jobs_rupd.as<RayUpdJob>() + step_off[s], n, mb, ctx->scan.vol, ctx->scan.alpha,
                             ctx->gmax, ctx->stream));
        continue;
      }
      KL(launch_bp_voxel(ctx->geom.as<ProjGeom>(), ctx->jobs_bp.as<BpJob>() + step_off[s], n, mb, ctx->scan.vol, W, H,
                         ctx->halfW, ctx->halfH, (float)ctx->scan.sdd, ctx->scan.ds, ctx->scan.alpha, ctx->gmax, 0,
                         exact, ctx->stream));
    }
  // max(vol * imROI, 0) over the whole volume, imROI == 1 (WaP_Tomo.cpp:1646-1659).
  bool contiguous = true;
  for (size_t q = 0; q < frames.size(); ++q) contiguous = contiguous && frames[q] == frames[0] + (int)q;
  if (contiguous && !frames.empty()) {
    KL(launch_roi_floor(ctx->nv * frames.size(), vol_ptr(ctx, frames[0]), ctx->stream));
  } else {
    for (int f : frames) KL(launch_roi_floor(ctx->nv, vol_ptr(ctx, f), ctx->stream));
  }
  return WAP_OK;
}

int ensure_world(wap_ctx *ctx) {
  const int *d = ctx->scan.vol;
  if (ctx->world.p) return WAP_OK;
  std::vector<float> h(d[0] + d[1] + d[2]);
  const float aabb[6] = {0, (float)d[0], 0, (float)d[1], 0, (float)d[2]};
  world_table(d, aabb, h.data());
  return upload(ctx, ctx->world, h);
}

// Warp-and-project for a set of frames, each at its s-th window projection
// (WaP_Tomo.cpp:796-822 driving WarpAndProjct, WaP_Tomo.cpp:1207-1421).
struct WapItem {
  int frame, proj;
  float rtime;
};

int wap_step(wap_ctx *ctx, const std::vector<WapItem> &items, int exact) {
  if (items.empty()) return WAP_OK;
  TRY(ensure_world(ctx));
  const size_t nv = ctx->nv, np = ctx->np;
  const int W = ctx->scan.det[0], H = ctx->scan.det[1];
  const int *d = ctx->scan.vol;
  const float aabb[6] = {0, (float)d[0], 0, (float)d[1], 0, (float)d[2]};
  const int nfames = ctx->F + 2;  // the level's frame list carries two padding copies
  std::vector<AdvectJob> fwd, adj;
  std::vector<FpJob> fp;
  std::vector<BpJob> bp;
  std::vector<AccJob> acc;
  for (const WapItem &it : items) {
    const int f = it.frame;
    const int ff = it.rtime < 0.0f ? std::max(0, f - 1) : std::min(nfames - 1, f);
    const int fa = std::max(0, f - 1);
    // A frame without a computed flow uses a zero field (flows start at zero).
    const float *vf = ff < ctx->F ? flow_ptr(ctx, ff) : ctx->zero_vol.as<float>();
    AdvectJob a{vf, vol_ptr(ctx, f), ctx->warped.as<float>() + (size_t)f * nv, it.rtime};
    fwd.push_back(a);
    FpJob j{};
    j.vol = a.out;
    j.proj = it.proj;
    j.meas = ctx->projs;
    j.dual = nullptr;
    j.corr = ctx->corr.as<float>() + (size_t)f * np;
    fp.push_back(j);
    BpJob b{};
    b.vol = ctx->delta.as<float>() + (size_t)f * nv;
    b.corr = j.corr;
    b.proj = it.proj;
    const int full[6] = {0, d[0], 0, d[1], 0, d[2]};
    std::memcpy(b.box, full, sizeof(full));
    bp.push_back(b);
    AdvectJob r{flow_ptr(ctx, fa), b.vol, ctx->back.as<float>() + (size_t)f * nv, -it.rtime};
    adj.push_back(r);
    acc.push_back(AccJob{vol_ptr(ctx, f), r.out});
  }
  std::vector<AdvectJob> advs = fwd;
  advs.insert(advs.end(), adj.begin(), adj.end());
  TRY(upload(ctx, ctx->jobs_adv, advs));
  TRY(upload(ctx, ctx->jobs_fp, fp));
  TRY(upload(ctx, ctx->jobs_bp, bp));
  TRY(upload(ctx, ctx->jobs_acc, acc));
  const int n = (int)items.size();
  const bool fast = ctx->flow_bits == 16;  // the precision form's warps
  const size_t bf = brick_floats(d);
  const bool bricks = ctx->fp_bricks != 0 && brick_room(ctx, bf * n);
  if (bricks) {  // the projector reads brick copies of the warped volumes
    std::vector<FpJob> fpb = fp;
    for (int q = 0; q < n; ++q) fpb[q].vol = ctx->bricks.as<float>() + q * bf;
    TRY(upload(ctx, ctx->jobs_fpb, fpb));
  }
  CU(ctx->adv_flags.ensure(sizeof(int) * 2 * n));
  KL(launch_advect(d, aabb, ctx->world.as<float>(), ctx->jobs_adv.as<AdvectJob>(), n, 1, ctx->stream, fast,
                   ctx->adv_flags.as<int>()));
  if (bricks) KL(launch_brick_jobs(ctx->jobs_fp.as<FpJob>(), n, ctx->bricks.as<float>(), d, ctx->stream, fast));
  KL(launch_forward(ctx->geom.as<ProjGeom>(), (bricks ? ctx->jobs_fpb : ctx->jobs_fp).as<FpJob>(), n, d, W, H, ctx->sd,
                    ctx->scan.alpha, ctx->stream, bricks, fast && bricks));
  ctx->stats.fp_launches++;
  for (const WapItem &it : items)
    CU(cudaMemsetAsync(ctx->delta.as<float>() + (size_t)it.frame * nv, 0, sizeof(float) * nv, ctx->stream));
  int mb[3] = {d[0], d[1], d[2]};
  KL(launch_bp_voxel(ctx->geom.as<ProjGeom>(), ctx->jobs_bp.as<BpJob>(), n, mb, d, W, H, ctx->halfW, ctx->halfH,
                     (float)ctx->scan.sdd, ctx->scan.ds, ctx->scan.alpha, ctx->gmax, 1, exact, ctx->stream));
  KL(launch_advect(d, aabb, ctx->world.as<float>(), ctx->jobs_adv.as<AdvectJob>() + n, n, 1, ctx->stream, fast,
                   ctx->adv_flags.as<int>() + n));
  ctx->stats.advect_voxels += 2.0 * n * (double)nv;
  ctx->stats.projections += n;
  ctx->stats.backprojections += n;
  KL(launch_wap_accumulate_batch(ctx->jobs_acc.as<AccJob>(), n, nv, ctx->scan.alpha, ctx->gmax, ctx->stream));
  return WAP_OK;
}

// PSART::AdaptiveWarp (WaP_Tomo.cpp:878-1204, commented out in the
// reference): per sweep, a zeroed delta volume; then for each projection of
// the frame's window in order, the forward projection of the volume warped by
// flow[max(0, f-1)] with the correction against one dual row (zeroed once per
// call), the bicubic backprojection added into the delta over the ROI box, and
// vol = cut(vol + alpha * warp(delta by flow[max(0, f-2)], -rtime), 0, G_Max);
// the delta keeps accumulating over the window.  At the end max(vol * imROI,
// 0).  rtime is the warp-and-project step's clamp((i - fTime) / tunit, -1, 1):
// the reference reads m_ProjIndex[i].rElapsed, a list it never fills.
int adaptive_warp(wap_ctx *ctx, int f, int nb_warp, int cut, int exact) {
  TRY(ensure_world(ctx));
  int box[6];
  TRY(roi_box(ctx, cut, box));
  const size_t nv = ctx->nv, np = ctx->np;
  const int W = ctx->scan.det[0], H = ctx->scan.det[1];
  const int *d = ctx->scan.vol;
  const float aabb[6] = {0, (float)d[0], 0, (float)d[1], 0, (float)d[2]};
  const int ff = std::max(0, f - 1), fa = std::max(0, f - 2);
  float *vol = vol_ptr(ctx, f);
  float *warped = ctx->warped.as<float>() + (size_t)f * nv, *delta = ctx->delta.as<float>() + (size_t)f * nv,
        *back = ctx->back.as<float>() + (size_t)f * nv;
  float *dual = ctx->dual.as<float>() + (size_t)f * ctx->maxwin * np, *corr = ctx->corr.as<float>() + (size_t)f * np;
  const int n = ctx->en[f] - ctx->st[f] + 1;
  std::vector<AdvectJob> adv;
  std::vector<FpJob> fp;
  std::vector<BpJob> bp;
  for (int i = ctx->st[f]; i <= ctx->en[f]; ++i) {
    float td = (i - ctx->ft[f]) / ctx->tunit;
    td = mac_min(mac_max(-1.0f, td), 1.0f);
    adv.push_back(AdvectJob{flow_ptr(ctx, ff), vol, warped, td});
    adv.push_back(AdvectJob{flow_ptr(ctx, fa), delta, back, -td});
    FpJob j{};
    j.vol = warped;
    j.proj = i;
    j.meas = ctx->projs;
    j.dual = dual;
    j.corr = corr;
    fp.push_back(j);
    BpJob b{};
    b.vol = delta;
    b.corr = corr;
    b.proj = i;
    std::memcpy(b.box, box, sizeof(box));
    bp.push_back(b);
  }
  TRY(upload(ctx, ctx->jobs_adv, adv));
  TRY(upload(ctx, ctx->jobs_fp, fp));
  TRY(upload(ctx, ctx->jobs_bp, bp));
  int mb[3] = {box[1] - box[0], box[3] - box[2], box[5] - box[4]};
  const bool fast = ctx->flow_bits == 16;
  CU(cudaMemsetAsync(dual, 0, sizeof(float) * np, ctx->stream));
  CU(ctx->adv_flags.ensure(sizeof(int) * 2));
  for (int it = 1; it <= nb_warp; ++it) {
    CU(cudaMemsetAsync(delta, 0, sizeof(float) * nv, ctx->stream));
    for (int q = 0; q < n; ++q) {
      KL(launch_advect(d, aabb, ctx->world.as<float>(), ctx->jobs_adv.as<AdvectJob>() + 2 * q, 1, 1, ctx->stream,
                       fast, ctx->adv_flags.as<int>()));
      KL(launch_forward(ctx->geom.as<ProjGeom>(), ctx->jobs_fp.as<FpJob>() + q, 1, d, W, H, ctx->sd, ctx->scan.alpha,
                        ctx->stream, false));
      KL(launch_bp_voxel(ctx->geom.as<ProjGeom>(), ctx->jobs_bp.as<BpJob>() + q, 1, mb, d, W, H, ctx->halfW,
                         ctx->halfH, (float)ctx->scan.sdd, ctx->scan.ds, ctx->scan.alpha, ctx->gmax, 1, exact,
                         ctx->stream));
      KL(launch_advect(d, aabb, ctx->world.as<float>(), ctx->jobs_adv.as<AdvectJob>() + 2 * q + 1, 1, 1, ctx->stream,
                       fast, ctx->adv_flags.as<int>() + 1));
      KL(launch_wap_accumulate(nv, vol, back, ctx->scan.alpha, ctx->gmax, ctx->stream, false));
      ctx->stats.fp_launches++;
      ctx->stats.projections++;
      ctx->stats.backprojections++;
      ctx->stats.advect_voxels += 2.0 * (double)nv;
    }
  }
  KL(launch_roi_floor(nv, vol, ctx->stream));
  return WAP_OK;
}

// ---------------------------------------------------------------------------
// Flow
// ---------------------------------------------------------------------------
int resize_tables(wap_ctx *ctx, int Sin, int Sout, ResizeTables &tb) {
  auto key = std::make_pair(Sin, Sout);
  auto it = ctx->resize_tables.find(key);
  if (it == ctx->resize_tables.end()) {
    HostResizeAxis h = make_resize_axis(Sin, Sout);
    std::unique_ptr<DevMem[]> m(new DevMem[6]);
    TRY(upload(ctx, m[0], h.tap_start));
    TRY(upload(ctx, m[1], h.tap_src));
    TRY(upload(ctx, m[2], h.tap_w));
    TRY(upload(ctx, m[3], h.base));
    // per output: t, t*t and (t*t)*t, the products the cubic's double
    // expression forms, computed once here in the same IEEE double
    std::vector<double> f3(3 * h.frac.size());
    for (size_t o = 0; o < h.frac.size(); ++o) {
      const double t = h.frac[o], t2 = t * t;
      f3[3 * o] = t;
      f3[3 * o + 1] = t2;
      f3[3 * o + 2] = t2 * t;
    }
    TRY(upload(ctx, m[4], f3));
    // the same weights as float pairs hi + lo (|w - (hi + lo)| <= 2^-48 |w|)
    // for the certified float-float growth
    std::vector<float> ff(2 * f3.size());
    for (size_t q = 0; q < f3.size(); ++q) {
      ff[2 * q] = (float)f3[q];
      ff[2 * q + 1] = (float)(f3[q] - (double)ff[2 * q]);
    }
    TRY(upload(ctx, m[5], ff));
    it = ctx->resize_tables.emplace(key, std::move(m)).first;
  }
  tb.tap_start = it->second[0].as<int>();
  tb.tap_src = it->second[1].as<int>();
  tb.tap_w = it->second[2].as<float>();
  tb.base = it->second[3].as<int>();
  tb.frac = it->second[4].as<double>();
  tb.frac_ff = it->second[5].as<float>();
  return WAP_OK;
}

int do_resize(wap_ctx *ctx, const int dims[3], int nc, const float *src, const int odims[3], float *out,
              bool fast = false) {
  const size_t big = (size_t)std::max(dims[0], odims[0]) * std::max(dims[1], odims[1]) *
                     std::max(dims[2], odims[2]) * nc;
  CU(ctx->rs_a.ensure(sizeof(float) * big));
  CU(ctx->rs_b.ensure(sizeof(float) * big));
  int cd[3] = {dims[0], dims[1], dims[2]};
  int axes[3], na = 0;
  for (int a = 0; a < 3; ++a)
    if (dims[a] != odims[a]) axes[na++] = a;
  if (na == 0) {
    CU(cudaMemcpyAsync(out, src, sizeof(float) * dims[0] * dims[1] * dims[2] * nc, cudaMemcpyDeviceToDevice,
                       ctx->stream));
    return WAP_OK;
  }
  const float *in = src;
  for (int q = 0; q < na; ++q) {
    const int a = axes[q];
    float *dst = (q == na - 1) ? out : ((q % 2 == 0) ? ctx->rs_a.as<float>() : ctx->rs_b.as<float>());
    ResizeTables tb;
    TRY(resize_tables(ctx, cd[a], odims[a], tb));
    KL(launch_resize_axis(a, cd, nc, odims[a], tb, in, dst, ctx->stream, fast));
    cd[a] = odims[a];
    in = dst;
  }
  return WAP_OK;
}

int do_blur(wap_ctx *ctx, const int dims[3], int nc, float sigma, const float *src, float *out) {
  const size_t n = (size_t)dims[0] * dims[1] * dims[2] * nc;
  const DericheCoefs k = deriche_coefs(sigma);
  int axes[3], na = 0;
  for (int a = 0; a < 3; ++a)
    if (dims[a] > 1) axes[na++] = a;
  if (k.skip || na == 0) {
    CU(cudaMemcpyAsync(out, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    return WAP_OK;
  }
  CU(ctx->blur_a.ensure(sizeof(float) * n));
  CU(ctx->blur_b.ensure(sizeof(float) * n));
  const float *in = src;
  for (int q = 0; q < na; ++q) {
    float *dst = (q == na - 1) ? out : ((q % 2 == 0) ? ctx->blur_a.as<float>() : ctx->blur_b.as<float>());
    KL(launch_deriche(axes[q], dims, nc, k, in, dst, ctx->stream));
    in = dst;
  }
  return WAP_OK;
}

FlowWork *flow_work(wap_ctx *ctx, const int dims[3]) {
  auto key = std::make_tuple(dims[0], dims[1], dims[2]);
  auto it = ctx->flow_work.find(key);
  if (it != ctx->flow_work.end()) return it->second.get();
  std::unique_ptr<FlowWork> w(new FlowWork);
  const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
  for (int a = 0; a < 3; ++a) w->n[a] = dims[a];
  if (w->va.ensure(sizeof(float) * 3 * nv) || w->vb.ensure(sizeof(float) * 3 * nv) ||
      w->y.ensure(sizeof(float) * 10 * nv) || w->y2.ensure(sizeof(float) * 10 * nv) ||
      w->u.ensure(sizeof(float) * 4 * nv) ||
      w->kty.ensure(sizeof(float) * 3 * nv) || w->kx4prev.ensure(sizeof(float) * nv) ||
      w->warp.ensure(sizeof(float) * nv) || w->acc.ensure(sizeof(double) * 2) || w->err.ensure(sizeof(float)) ||
      w->world.ensure(sizeof(float) * (dims[0] + dims[1] + dims[2])))
    return nullptr;
  FlowWork *p = w.get();
  ctx->flow_work.emplace(key, std::move(w));
  return p;
}

// The primal-dual iteration's kernel form and z-chunk for one grid: the
// fused kernel or the primal + dual pair, each over a few z-chunks.  Both
// forms compute identical bits, so the choice changes only speed.  Unless
// forced (wap_set_tuning), the candidates are timed once per grid size with
// CUDA events on the context's stream; a candidate launch only reads the
// current iterate and writes the next-iterate buffers, which the real
// iteration then overwrites, so tuning leaves the solver's state untouched.
template <class Launch>
int pd_plan(wap_ctx *ctx, const FlowDims &D, Launch &launch, int &form, int &zchunk, bool tma, bool half = false) {
  const int *n = D.n;
  const auto key = std::make_tuple(n[0], n[1], n[2]);
  auto &plans = half ? ctx->pd_plans16 : ctx->pd_plans;
  // z-chunk defaults: about 4 waves of 2 fused blocks / 8 waves of 6 split
  // blocks over the 152 SMs.
  const int tiles_f = ((n[0] + 31) / 32) * ((n[1] + 6) / 7);
  const int tiles_s = ((n[0] + 31) / 32) * ((n[1] + 7) / 8);
  const int zf = std::max(2, std::min(64, n[2] * tiles_f / 1216));
  const int zs = std::max(2, std::min(32, n[2] * tiles_s / 7296));
  const int zt = std::max(4, std::min(64, n[2] * tiles_s / 1216));
  if (half) {  // FP16 storage exists only in the TMA form (form 4)
    if (ctx->pd_zchunk) {
      form = 4;
      zchunk = ctx->pd_zchunk;
      return WAP_OK;
    }
  } else if (ctx->pd_form) {
    form = ctx->pd_form == 3 && !tma ? 2 : ctx->pd_form;
    zchunk = ctx->pd_zchunk ? ctx->pd_zchunk : (form == 1 ? zf : form == 2 ? zs : zt);
    return WAP_OK;
  }
  auto it = plans.find(key);
  if (it != plans.end()) {
    form = it->second.first;
    zchunk = it->second.second;
    return WAP_OK;
  }
  const auto gkey = std::make_tuple(ctx->device, n[0], n[1], n[2], half ? 1 : 0, tma ? 1 : 0);
  {
    std::lock_guard<std::mutex> lk(g_plan_mutex);
    auto g = g_plans.find(gkey);
    if (g != g_plans.end()) {
      plans[key] = g->second;
      form = g->second.first;
      zchunk = g->second.second;
      return WAP_OK;
    }
  }
  std::vector<std::pair<int, int>> cand;
  // TMA-form chunks: the kernel time is flat within a few per cent from about
  // a quarter to half of zt (short chunks repeat a plane's primal, long ones
  // leave a partial last wave), so the candidates span zt/4..zt, plus the two
  // chunk lengths (4..64 planes) whose chunk counts come closest to filling
  // whole waves of resident blocks (the kernel balances the chunk lengths).
  std::vector<int> zts = {zt / 4, zt / 3, zt / 2, zt};
  if (tma || half) {
    const int slots = pd_tma_slots(half), tiles = pd_tma_tiles(D);
    std::vector<std::pair<double, int>> waves;  // (-wave fill, rounded; z-chunk)
    for (int nc = 1; slots > 0 && nc <= n[2] / 4; ++nc) {
      const int z = (n[2] + nc - 1) / nc;
      if ((n[2] + z - 1) / z != nc || z > 64) continue;  // not a grid of nc chunks
      const double w = (double)tiles * nc / slots, fill = w / std::ceil(w);
      if (fill >= 0.96) waves.emplace_back(-std::round(fill * 100.0) - std::fabs(z - zt / 2.0) * 1e-3, z);
    }
    std::sort(waves.begin(), waves.end());
    for (size_t q = 0; q < waves.size() && q < 2; ++q)
      if (std::find(zts.begin(), zts.end(), waves[q].second) == zts.end()) zts.push_back(waves[q].second);
  }
  if (half) {
    for (int z : zts)
      if (z >= 2 && z <= n[2] && (cand.empty() || cand.back().second != z)) cand.emplace_back(4, z);
    if (cand.empty()) cand.emplace_back(4, std::max(1, n[2]));
  } else {
    for (int z : {zf / 2, zf, zf * 2})
      if (z >= 1 && z <= n[2]) cand.emplace_back(1, z);
    for (int z : {zs / 2, zs, zs * 2, zs * 4})
      if (z >= 1 && z <= n[2]) cand.emplace_back(2, z);
    if (tma)
      for (int z : zts)
        if (z >= 2 && z <= n[2] && (cand.back().first != 3 || cand.back().second != z)) cand.emplace_back(3, z);
  }
  ScopedEvents ev(2);
  CU(ev.create());
  const cudaEvent_t e0 = ev[0], e1 = ev[1];
  float best = 1e30f;
  std::pair<int, int> pick = cand.front();
  for (const auto &c : cand) {
    KL(launch(c.first, c.second, 0, 0, 0));  // warm-up
    CU(cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < 3; ++r) KL(launch(c.first, c.second, 0, 0, 0));
    CU(cudaEventRecord(e1, ctx->stream));
    CU(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CU(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  plans[key] = pick;
  {
    std::lock_guard<std::mutex> lk(g_plan_mutex);
    g_plans[gkey] = pick;
  }
  form = pick.first;
  zchunk = pick.second;
  return WAP_OK;
}

// optical_flow::L1TVOpticalFlowNonlinear3D (optical_flow.h:88-995).
// V (3 ch) is read and written whole; Y (10 ch: Y1,Y2,Y3,Y4) is read whole
// and written on the ROI only, as the reference writes back.
int flow_level(wap_ctx *ctx, const int dims[3], const float *I1, const float *I2, float *V, float *Y[4], float tol,
               float lambda, int max_iters, int nwarps, const float aabb[6], const int roi6[6], int *iters_out,
               long long *total) {
  // The primal-dual kernels index the 10-component dual with 32-bit offsets.
  CHECK(10ull * dims[0] * dims[1] * dims[2] < (1ull << 32), WAP_ETOOBIG,
        "flow grid too large for 32-bit offsets (under 2^32/10 voxels)");
  FlowWork *w = flow_work(ctx, dims);
  CHECK(w, WAP_ENOMEM, "flow workspace allocation failed");
  const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
  FlowDims D;
  for (int a = 0; a < 3; ++a) D.n[a] = dims[a];
  for (int a = 0; a < 6; ++a) D.roi[a] = roi6[a];
  // world table for this grid and box
  if (std::memcmp(w->aabb_key, aabb, sizeof(w->aabb_key)) != 0 || !w->world.p) {
    std::vector<float> h(dims[0] + dims[1] + dims[2]);
    world_table(dims, aabb, h.data());
    CU(cudaMemcpyAsync(w->world.p, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    std::memcpy(w->aabb_key, aabb, sizeof(w->aabb_key));
  }
  float *vcur = w->va.as<float>(), *vnext = w->vb.as<float>();
  float *y = w->y.as<float>();
  float *ycur = y, *ynext = w->y2.as<float>();
  CU(cudaMemcpyAsync(vcur, V, sizeof(float) * 3 * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  CU(cudaMemcpyAsync(vnext, V, sizeof(float) * 3 * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  for (int q = 0; q < 3; ++q)
    CU(cudaMemcpyAsync(y + 3 * q * nv, Y[q], sizeof(float) * 3 * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  CU(cudaMemcpyAsync(y + 9 * nv, Y[3], sizeof(float) * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  CU(cudaMemsetAsync(w->u.p, 0, sizeof(float) * 4 * nv, ctx->stream));
  CU(cudaMemsetAsync(w->kty.p, 0, sizeof(float) * 3 * nv, ctx->stream));
  const float sigma1 = std::min(1.0f / 3.0f, std::min(1.0f / 3.0f, 1.0f / 3.0f));
  double *acc = w->acc.as<double>();
  // The dual's shrink divides by the constant lambda + 2 sigma1; the FMA-
  // corrected reciprocal is used only once it is proven bit-identical to IEEE
  // division for this constant over all 2^32 inputs.
  const float den = lambda + 2 * sigma1;
  const float rinv = 1.0f / den;
  uint32_t den_bits;
  std::memcpy(&den_bits, &den, 4);
  // Proofs are per device and shared by every context in the process
  // (key 0: the reciprocal; otherwise the divisor's bits).
  auto proven = [&](uint64_t key, float dv, int &out) -> int {
    {
      std::lock_guard<std::mutex> lk(g_proof_mutex);
      auto it = g_proofs.find(std::make_pair(ctx->device, key));
      if (it != g_proofs.end()) {
        out = it->second;
        return WAP_OK;
      }
    }
    DevMem bad;
    CU(bad.ensure(sizeof(unsigned long long)));
    if (key == 0) KL(launch_pd_rcp_check(bad.as<unsigned long long>(), ctx->stream));
    else KL(launch_pd_fastdiv_check(dv, 1.0f / dv, bad.as<unsigned long long>(), ctx->stream));
    unsigned long long nbad = 1;
    CU(cudaMemcpyAsync(&nbad, bad.p, sizeof(nbad), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    out = nbad == 0 ? 1 : 0;
    std::lock_guard<std::mutex> lk(g_proof_mutex);
    g_proofs[std::make_pair(ctx->device, key)] = out;
    return WAP_OK;
  };
  // fastdiv bit 0: the shrink's divisor den; bit 1: the residual's sigma1
  // (the TMA form's residual iterations divide nine dual terms by it)
  int fastdiv = 0, fast_s = 0, rcp = 0;
  uint32_t s1_bits;
  std::memcpy(&s1_bits, &sigma1, 4);
  TRY(proven(((uint64_t)1 << 32) | den_bits, den, fastdiv));
  TRY(proven(((uint64_t)1 << 32) | s1_bits, sigma1, fast_s));
  TRY(proven(0, 0.0f, rcp));
  fastdiv |= fast_s << 1;
  int form = 0, zchunk = 0;
  if (w->tma_state == 0) {
    w->tma_state = -1;
    if (pd_tma_supported(D, false) && w->tma_err.ensure(sizeof(int)) == cudaSuccess &&
        make_pd_tma_maps(D, false, w->y.p, w->u.p, w->va.p, &w->ymap[0], &w->umap, &w->vmap[0]) == cudaSuccess &&
        make_pd_tma_maps(D, false, w->y2.p, w->u.p, w->vb.p, &w->ymap[1], &w->umap, &w->vmap[1]) == cudaSuccess) {
      w->tma_state = 1;
      CU(cudaMemsetAsync(w->tma_err.p, 0, sizeof(int), ctx->stream));
    }
  }
  // The precision form: y, v, u live in FP16 copies during the iterations
  // (FP32 arithmetic); the FP32 buffers are refreshed where the rest of the
  // solver reads them (before each warp's advection and at the end).
  if (ctx->flow_bits == 16 && w->h_state == 0) {
    w->h_state = -1;
    if (pd_tma_supported(D, true) && w->tma_err.ensure(sizeof(int)) == cudaSuccess &&
        w->yh[0].ensure(4 * 5 * nv) == cudaSuccess && w->yh[1].ensure(4 * 5 * nv) == cudaSuccess &&
        w->vh[0].ensure(4 * 2 * nv) == cudaSuccess && w->vh[1].ensure(4 * 2 * nv) == cudaSuccess &&
        w->uh.ensure(2 * 4 * nv) == cudaSuccess &&
        make_pd_tma_maps(D, true, w->yh[0].p, w->uh.p, w->vh[0].p, &w->hymap[0], &w->humap, &w->hvmap[0]) ==
            cudaSuccess &&
        make_pd_tma_maps(D, true, w->yh[1].p, w->uh.p, w->vh[1].p, &w->hymap[1], &w->humap, &w->hvmap[1]) ==
            cudaSuccess) {
      w->h_state = 1;
      CU(cudaMemsetAsync(w->tma_err.p, 0, sizeof(int), ctx->stream));
    }
  }
  const bool half = ctx->flow_bits == 16 && w->h_state == 1;
  if (half) {
    KL(launch_to_pairs(nv, 10, y, w->yh[0].p, ctx->stream));
    KL(launch_to_pairs(nv, 3, w->va.as<float>(), w->vh[0].p, ctx->stream));
    KL(launch_to_pairs(nv, 3, w->vb.as<float>(), w->vh[1].p, ctx->stream));
  }
  auto pd_launch = [&](int f, int zc, int mode, int store, int res) -> cudaError_t {
    const int yi = ycur == w->y.as<float>() ? 0 : 1, vi = vcur == w->va.as<float>() ? 0 : 1;
    if (f == 4)
      return launch_pd_tma(D, zc, true, &w->hymap[yi], &w->humap, &w->hvmap[vi], w->yh[1 - yi].p,
                           w->vh[1 - vi].p, w->kty.as<float>(), w->kx4prev.as<float>(), mode, lambda, sigma1, rinv,
                           fastdiv, rcp, store, res, acc, w->tma_err.as<int>(), ctx->stream);
    if (f == 3)
      return launch_pd_tma(D, zc, false, &w->ymap[yi], &w->umap, &w->vmap[vi], ynext, vnext, w->kty.as<float>(),
                           w->kx4prev.as<float>(), mode, lambda, sigma1, rinv, fastdiv, rcp, store, res, acc,
                           w->tma_err.as<int>(), ctx->stream);
    if (f == 1)
      return launch_pd_fused(D, zc, ycur, ynext, w->u.as<float>(), vcur, vnext, w->kty.as<float>(),
                             w->kx4prev.as<float>(), mode, lambda, sigma1, rinv, fastdiv, rcp, store, res, acc,
                             ctx->stream);
    return launch_pd_split(D, zc, ycur, ynext, w->u.as<float>(), vcur, vnext, w->kty.as<float>(),
                           w->kx4prev.as<float>(), mode, lambda, sigma1, rinv, fastdiv, rcp, store, res, acc,
                           ctx->stream);
  };
  AdvectJob aj{vcur, I2, w->warp.as<float>(), -1.0f};
  for (int wi = 0; wi < nwarps; ++wi) {
    // advect I2 by the current flow, dt = -1 (optical_flow.h:418)
    aj.vel = vcur;
    std::vector<AdvectJob> ajs{aj};
    TRY(upload(ctx, ctx->jobs_misc, ajs));
    CU(ctx->adv_flags.ensure(sizeof(int) * 2));
    KL(launch_advect(dims, aabb, w->world.as<float>(), ctx->jobs_misc.as<AdvectJob>(), 1, 1, ctx->stream,
                     ctx->flow_bits == 16, ctx->adv_flags.as<int>()));
    ctx->stats.advect_voxels += (double)nv;
    KL(launch_linearize(D, w->warp.as<float>(), I1, vcur, w->u.as<float>(), w->kx4prev.as<float>(), ctx->stream));
    if (half) KL(launch_to_pairs(nv, 4, w->u.as<float>(), w->uh.p, ctx->stream));
    if (wi == 0 && max_iters >= 0) {
      TRY(pd_plan(ctx, D, pd_launch, form, zchunk, w->tma_state == 1, half));
      if (w->tma_state == 1 || half) {  // a tuning launch of the TMA form must not have timed out either
        int bad = 0;
        CU(cudaMemcpyAsync(&bad, w->tma_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        CHECK(bad == 0, WAP_ECUDA, "primal-dual TMA pipeline: a barrier wait timed out");
      }
    }
    int it = 0;
    float err = 1.0f;
    // Profile only the largest grid seen in this outer iteration.
    const bool prof = ctx->profiling && (long long)nv >= ctx->stats.pd_timed_voxels;
    if (prof && (long long)nv > ctx->stats.pd_timed_voxels) {
      ctx->stats.pd_timed_voxels = (long long)nv;
      ctx->stats.ms_pd = 0.0;
      ctx->stats.pd_timed = 0;
    }
    int pending = 0;
    auto drain = [&]() -> int {
      for (int q = 0; q < pending; ++q) {
        float ms = 0.0f;
        CU(cudaEventElapsedTime(&ms, ctx->pd_events[2 * q], ctx->pd_events[2 * q + 1]));
        ctx->stats.ms_pd += ms;
        ctx->stats.pd_timed++;
      }
      pending = 0;
      return WAP_OK;
    };
    while (err > tol && it <= max_iters) {
      ++it;
      const int res = (it % 50 == 0);
      const int store = ((it + 1) % 50 == 0);
      if (res) CU(cudaMemsetAsync(acc, 0, sizeof(double) * 2, ctx->stream));
      // Timed launches: every tenth, so that the events between launches
      // leave the others free to overlap their start with the previous
      // grid's tail (programmatic dependent launch).
      const bool timed = prof && pending < 50 && it % 10 == 3;
      if (timed) CU(cudaEventRecord(ctx->pd_events[2 * pending], ctx->stream));
      const int mode = (it == 1) ? (wi == 0 ? 1 : 2) : 0;
      KL(pd_launch(form, zchunk, mode, store, res));
      if (timed) CU(cudaEventRecord(ctx->pd_events[2 * pending++ + 1], ctx->stream));
      std::swap(vcur, vnext);
      std::swap(ycur, ynext);
      if (res) {
        KL(launch_residual_finish(acc, (int)nv, w->err.as<float>(), ctx->stream));
        CU(cudaMemcpyAsync(&err, w->err.p, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        TRY(drain());
      }
    }
    if (pending) {
      CU(cudaStreamSynchronize(ctx->stream));
      TRY(drain());
    }
    if (half) KL(launch_from_pairs(nv, 3, w->vh[vcur == w->va.as<float>() ? 0 : 1].p, vcur, ctx->stream));
    if (form >= 3) {
      int bad = 0;
      CU(cudaMemcpyAsync(&bad, w->tma_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      CU(cudaStreamSynchronize(ctx->stream));
      CHECK(bad == 0, WAP_ECUDA, "primal-dual TMA pipeline: a barrier wait timed out");
    }
    ctx->stats.pd_voxel_iters += (double)it * (double)nv;
    if (iters_out) iters_out[wi] = it;
    if (total) *total += it;
    ctx->stats.flow_pd_iterations += it;
  }
  if (half) KL(launch_from_pairs(nv, 10, w->yh[ycur == w->y.as<float>() ? 0 : 1].p, ycur, ctx->stream));
  CU(cudaMemcpyAsync(V, vcur, sizeof(float) * 3 * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  for (int q = 0; q < 3; ++q) KL(launch_roi_copy(D, 3, ycur + 3 * q * nv, Y[q], ctx->stream));
  KL(launch_roi_copy(D, 1, ycur + 9 * nv, Y[3], ctx->stream));
  return WAP_OK;
}

int flow_multiscale(wap_ctx *ctx, const int dims[3], const float *I1, const float *I2, const float *V0, float tol,
                    float lambda, int max_iters, int nwarps, float eta, float sigma, int scales, const int cut6[6],
                    float *Vout, long long *total, const float *const *Y0 = nullptr) {
  CHECK(scales >= 1 && scales <= 16, WAP_EINVAL, "scales out of range");
  const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
  // blurred inputs live in the two finest-level image buffers' sources
  std::vector<int> ld(3 * scales);
  float t_eta = 1.0f;
  for (int s = 0; s < scales; ++s) {
    const int l = scales - 1 - s;  // coarse first
    for (int a = 0; a < 3; ++a) ld[3 * l + a] = (int)(dims[a] * t_eta);
    for (int a = 0; a < 3; ++a) CHECK(ld[3 * l + a] >= 3, WAP_EINVAL, "pyramid level smaller than 3 voxels");
    t_eta = t_eta * eta;
  }
  if ((int)ctx->pyramid.size() < scales) ctx->pyramid.resize(scales);
  for (int l = 0; l < scales; ++l) {
    if (!ctx->pyramid[l]) ctx->pyramid[l].reset(new PyramidLevel);
    PyramidLevel &P = *ctx->pyramid[l];
    for (int a = 0; a < 3; ++a) P.d[a] = ld[3 * l + a];
    const size_t m = (size_t)P.d[0] * P.d[1] * P.d[2];
    CU(P.i1.ensure(sizeof(float) * m));
    CU(P.i2.ensure(sizeof(float) * m));
    CU(P.v.ensure(sizeof(float) * 3 * m));
    CU(P.y.ensure(sizeof(float) * 10 * m));
  }
  // blur at full resolution, then build the pyramid (optical_flow.h:1010-1052)
  PyramidLevel &fine = *ctx->pyramid[scales - 1];
  DevMem &b1 = ctx->pyr_b1, &b2 = ctx->pyr_b2;  // persistent: no allocation (and no free) per pair
  CU(b1.ensure(sizeof(float) * nv));
  CU(b2.ensure(sizeof(float) * nv));
  TRY(do_blur(ctx, dims, 1, sigma, I1, b1.as<float>()));
  TRY(do_blur(ctx, dims, 1, sigma, I2, b2.as<float>()));
  for (int l = 0; l < scales; ++l) {
    PyramidLevel &P = *ctx->pyramid[l];
    TRY(do_resize(ctx, dims, 1, b1.as<float>(), P.d, P.i1.as<float>()));
    TRY(do_resize(ctx, dims, 1, b2.as<float>(), P.d, P.i2.as<float>()));
  }
  // Only the coarsest level starts from the arguments: every finer level's
  // V and Y are replaced by the upsampled result of the level below
  // (optical_flow.h:1101-1115) before they are used.
  {
    PyramidLevel &P = *ctx->pyramid[0];
    const size_t m = (size_t)P.d[0] * P.d[1] * P.d[2];
    TRY(do_resize(ctx, dims, 3, V0, P.d, P.v.as<float>()));
    if (Y0) {
      TRY(do_resize(ctx, dims, 3, Y0[0], P.d, P.y.as<float>()));
      TRY(do_resize(ctx, dims, 3, Y0[1], P.d, P.y.as<float>() + 3 * m));
      TRY(do_resize(ctx, dims, 3, Y0[2], P.d, P.y.as<float>() + 6 * m));
      TRY(do_resize(ctx, dims, 1, Y0[3], P.d, P.y.as<float>() + 9 * m));
    } else {
      CU(cudaMemsetAsync(P.y.p, 0, sizeof(float) * 10 * m, ctx->stream));
    }
  }
  const float aabb[6] = {0, (float)dims[0], 0, (float)dims[1], 0, (float)dims[2]};
  ScopedEvents lev(scales + 1);
  CU(lev.create());
  CU(cudaEventRecord(lev[0], ctx->stream));
  for (int l = 0; l < scales; ++l) {
    PyramidLevel &P = *ctx->pyramid[l];
    const size_t m = (size_t)P.d[0] * P.d[1] * P.d[2];
    int roi[6];
    for (int i = 0; i < 6; ++i) roi[i] = (float)cut6[i] * ((float)P.d[i / 2] / (float)dims[i / 2]);
    float *Y[4] = {P.y.as<float>(), P.y.as<float>() + 3 * m, P.y.as<float>() + 6 * m, P.y.as<float>() + 9 * m};
    long long before = total ? *total : 0, its = 0;
    TRY(flow_level(ctx, P.d, P.i1.as<float>(), P.i2.as<float>(), P.v.as<float>(), Y, tol, lambda, max_iters, nwarps,
                   aabb, roi, nullptr, &its));
    if (total) *total = before + its;
    const int fine_idx = scales - 1 - l;  // 0 = finest
    if (fine_idx < 8) ctx->stats.pd_iters_level[fine_idx] += its;
    CU(cudaEventRecord(lev[l + 1], ctx->stream));
    if (l + 1 < scales) {
      PyramidLevel &N = *ctx->pyramid[l + 1];
      // the precision form grows the flow and the dual in float
      const bool fast = ctx->flow_bits == 16;
      TRY(do_resize(ctx, P.d, 3, P.v.as<float>(), N.d, N.v.as<float>(), fast));
      TRY(do_resize(ctx, P.d, 10, P.y.as<float>(), N.d, N.y.as<float>(), fast));
    }
  }
  CU(cudaMemcpyAsync(Vout, fine.v.p, sizeof(float) * 3 * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  for (int l = 0; l < scales; ++l) {
    float ms = 0.0f;
    CU(cudaEventElapsedTime(&ms, lev[l], lev[l + 1]));
    if (scales - 1 - l < 8) ctx->stats.ms_flow_level[scales - 1 - l] += ms;
  }
  return WAP_OK;
}

int check_schedule(wap_ctx *ctx, const wap_schedule *sch, int f0, int f1) {
  CHECK(ctx && sch, WAP_EINVAL, "null argument");
  CHECK(ctx->level >= 0, WAP_ESTATE, "no level set up");
  CHECK(ctx->projs, WAP_ESTATE, "no projections uploaded");
  CHECK(0 <= f0 && f0 < f1 && f1 <= ctx->F, WAP_EINVAL, "frame range out of bounds");
  CHECK(sch->cut >= 1 && 2 * sch->cut < ctx->scan.vol[0] && 2 * sch->cut < ctx->scan.vol[1] &&
            2 * sch->cut < ctx->scan.vol[2],
        WAP_EINVAL, "cut must leave a non-empty ROI and be at least 1");
  CHECK(sch->n_cp >= 0 && sch->nb_sart >= 0 && sch->nb_projwarp >= 0 && sch->flow_iters >= 0 &&
            sch->flow_warps >= 0 && sch->flow_scales >= 1,
        WAP_EINVAL, "negative schedule count");
  return WAP_OK;
}

// One CP iteration (number icp, 1-based) over frames [f0, f1): dual, primal,
// SART proximal operator, over-relaxation (WaP_Tomo.cpp:563-690), each
// batched over the frames.
int cp_pass(wap_ctx *ctx, const wap_schedule *sch, int f0, int f1, int icp) {
  int box[6];
  roi_box(ctx, sch->cut, box);
  CpArgs ca;
  for (int a = 0; a < 3; ++a) ca.n[a] = ctx->scan.vol[a];
  std::memcpy(ca.box, box, sizeof(box));
  ca.f0 = f0;
  ca.F = f1 - f0;
  ca.Ftot = ctx->F;
  ca.sigma = (float)(.9 / (8.0f * 1.0f));
  ca.tau = 1.0f;
  ca.tv_w = (float)ctx->scan.tv_w;
  ca.tp_w = (float)ctx->scan.tp_w;
  ca.gmax = ctx->gmax;
  std::vector<int> frames;
  for (int f = f0; f < f1; ++f) frames.push_back(f);
  KL(launch_cp_dual(ca, ctx->xbar.as<float>(), ctx->zero_vol.as<float>(), ctx->ytv.as<float>(),
                    ctx->ytp.as<float>(), ctx->stream));
  KL(launch_cp_primal(ca, ctx->ytp.as<float>(), ctx->ytv.as<float>(), ctx->vols.as<float>(), ctx->xprev.as<float>(),
                      ctx->stream));
  TRY(sart_frames(ctx, frames, sch->nb_sart, box, sch->bp_exact));
  for (int f : frames) TRY(notify(ctx, WAP_EV_SART, f, icp, vol_ptr(ctx, f)));
  KL(launch_cp_overrelax(ca, ctx->vols.as<float>(), ctx->xprev.as<float>(), ctx->xbar.as<float>(), ctx->stream));
  ctx->stats.cp_frame_passes += ca.F;
  return WAP_OK;
}

// The multiscale flow of the pair (f, f+1) (WaP_Tomo.cpp:732-777).
int flow_pair(wap_ctx *ctx, const wap_schedule *sch, int f) {
  const int cut6[6] = {sch->cut, sch->cut, sch->cut, sch->cut, sch->cut, sch->cut};
  long long total = 0;
  TRY(flow_multiscale(ctx, ctx->scan.vol, vol_ptr(ctx, f), vol_ptr(ctx, f + 1), flow_ptr(ctx, f), sch->flow_tol,
                      sch->flow_lambda, sch->flow_iters, sch->flow_warps, sch->flow_eta, sch->flow_sigma,
                      sch->flow_scales, cut6, flow_ptr(ctx, f), &total));
  TRY(notify(ctx, WAP_EV_FLOW, f, 0, flow_ptr(ctx, f)));
  return WAP_OK;
}

void merge_flow_stats(wap_stats &d, const wap_stats &s) {
  d.flow_pd_iterations += s.flow_pd_iterations;
  d.kernel_launches += s.kernel_launches;
  d.pd_voxel_iters += s.pd_voxel_iters;
  d.advect_voxels += s.advect_voxels;
  for (int l = 0; l < 8; ++l) {
    d.ms_flow_level[l] += s.ms_flow_level[l];
    d.pd_iters_level[l] += s.pd_iters_level[l];
  }
  if (s.pd_timed_voxels > d.pd_timed_voxels) {
    d.pd_timed_voxels = s.pd_timed_voxels;
    d.ms_pd = s.ms_pd;
    d.pd_timed = s.pd_timed;
  } else if (s.pd_timed_voxels == d.pd_timed_voxels) {
    d.ms_pd += s.ms_pd;
    d.pd_timed += s.pd_timed;
  }
}

// The flow pairs of frames [f0, f1) (WaP_Tomo.cpp:732-777).  A pair reads two
// frames' volumes and writes its own flow, so the pairs are independent: with
// flow_lanes > 1 they run concurrently, each lane a helper compute context
// with its own stream and flow workspaces, fed by its own host thread and
// taking the next pair from a shared counter.  While one pair's finest level
// streams from HBM, another's coarse levels and 128^3 level, latency-bound
// on their own, fill the gaps.  Each pair's flow is the one it gets alone.
// The pairs run in turn when an observer is set (its events come in pair
// order), when one pair is due, and the first time a flow shape is seen, so
// that the autotuner times its candidates undisturbed.
// Automatic lane count: measured outer iterations (16 frames, fixed 3000
// primal-dual iterations per warp and level) with 2 / 4 lanes: 64^3 2.01 /
// 1.57 s, 96^3 4.60 / 4.46 s, 128^3 8.45 / 8.23 s; at 256^3 two lanes, whose
// finest levels stream from HBM, are as fast as three.
constexpr size_t kAutoLanesSmallVoxels = (size_t)128 * 128 * 128;
constexpr int kAutoLanesSmall = 4;

int flow_phase(wap_ctx *ctx, const wap_schedule *sch, int f0, int f1) {
  std::vector<int> pairs;
  for (int f = f0; f < f1 && f + 1 < ctx->F; ++f) pairs.push_back(f);
  const auto shape = std::make_tuple(ctx->scan.vol[0], ctx->scan.vol[1], ctx->scan.vol[2], sch->flow_scales,
                                     ctx->flow_bits, (int)std::lround(sch->flow_eta * 1e6));
  size_t first = 0;
  if (!ctx->lanes_tuned.count(shape) && !pairs.empty()) {
    TRY(flow_pair(ctx, sch, pairs[0]));
    ctx->lanes_tuned.insert(shape);
    first = 1;
  }
  const size_t nv = (size_t)ctx->scan.vol[0] * ctx->scan.vol[1] * ctx->scan.vol[2];
  const int lanes = ctx->flow_lanes > 0 ? ctx->flow_lanes : nv <= kAutoLanesSmallVoxels ? kAutoLanesSmall : 2;
  const int K = std::min<int>(lanes, (int)(pairs.size() - first));
  if (K <= 1 || ctx->observer) {
    for (size_t i = first; i < pairs.size(); ++i) TRY(flow_pair(ctx, sch, pairs[i]));
    return WAP_OK;
  }
  while ((int)ctx->lanes.size() < K) {
    wap_ctx *h = nullptr;
    const int r = wap_create_compute(&h, ctx->device);
    CHECK(r == WAP_OK, r, "flow lane: context creation failed");
    ctx->lanes.push_back(h);
  }
  for (int q = 0; q < K; ++q) {  // the settings the pairs run with
    wap_ctx *h = ctx->lanes[q];
    h->flow_bits = ctx->flow_bits;
    h->pd_form = ctx->pd_form;
    h->pd_zchunk = ctx->pd_zchunk;
    h->pd_plans.clear();  // refilled from the process-wide plans
    h->pd_plans16.clear();
    if (ctx->profiling && h->pd_events.empty()) {
      const int r = wap_set_profiling(h, 1);
      CHECK(r == WAP_OK, r, "flow lane: " + h->err);
    }
    h->profiling = ctx->profiling;
    h->stats = wap_stats{};
  }
  // the lanes start after the work enqueued so far (the volumes the pairs read)
  ScopedEvents ev(1 + K);
  CU(ev.create());
  CU(cudaEventRecord(ev[0], ctx->stream));
  for (int q = 0; q < K; ++q) CU(cudaStreamWaitEvent(ctx->lanes[q]->stream, ev[0], 0));
  const int cut6[6] = {sch->cut, sch->cut, sch->cut, sch->cut, sch->cut, sch->cut};
  std::atomic<size_t> next{first};
  std::atomic<bool> failed{false};  // a lane's error: the others take no further pair
  std::vector<int> rcs(K, WAP_OK);
  auto lane = [&](int q) {
    wap_ctx *h = ctx->lanes[q];
    try {
      if (cudaSetDevice(ctx->device) != cudaSuccess) {
        rcs[q] = fail(h, WAP_ECUDA, "cudaSetDevice failed");
        failed = true;
        return;
      }
      for (size_t i; !failed && (i = next.fetch_add(1)) < pairs.size();) {
        const int f = pairs[i];
        long long total = 0;
        const int r = flow_multiscale(h, ctx->scan.vol, vol_ptr(ctx, f), vol_ptr(ctx, f + 1), flow_ptr(ctx, f),
                                      sch->flow_tol, sch->flow_lambda, sch->flow_iters, sch->flow_warps,
                                      sch->flow_eta, sch->flow_sigma, sch->flow_scales, cut6, flow_ptr(ctx, f),
                                      &total);
        if (r != WAP_OK) {
          rcs[q] = r;
          failed = true;
          return;
        }
      }
    } catch (const std::bad_alloc &) {
      rcs[q] = fail(h, WAP_ENOMEM, "out of memory");  // short: no allocation
      failed = true;
    } catch (...) {
      rcs[q] = fail(h, WAP_EHOST, "host exception");
      failed = true;
    }
  };
  std::vector<std::thread> th;
  int started = 1;
  try {
    th.reserve(K - 1);
    for (; started < K; ++started) th.emplace_back(lane, started);
  } catch (...) {  // no more threads: fewer lanes (the counter hands them the pairs)
  }
  lane(0);
  for (auto &t : th) t.join();
  for (int q = 0; q < K; ++q) {
    if (q < started) {
      CU(cudaEventRecord(ev[1 + q], ctx->lanes[q]->stream));
      CU(cudaStreamWaitEvent(ctx->stream, ev[1 + q], 0));
    }
    merge_flow_stats(ctx->stats, ctx->lanes[q]->stats);
  }
  for (int q = 0; q < K; ++q)
    if (rcs[q] != WAP_OK) return fail(ctx, rcs[q], "flow lane " + std::to_string(q) + ": " + ctx->lanes[q]->err);
  return WAP_OK;
}

// Warp-and-project over the windows of the visited frames in [f0, f1)
// (WaP_Tomo.cpp:796-822), batched over frames by window slot.
int wap_pass(wap_ctx *ctx, const wap_schedule *sch, int f0, int f1) {
  const int wend = std::min(f1, std::min(sch->wp_frames, ctx->F));
  int maxnum = 0;
  for (int f = f0; f < wend; ++f) maxnum = std::max(maxnum, ctx->en[f] - ctx->st[f] + 1);
  for (int wp = 0; wp < sch->nb_projwarp; ++wp)
    for (int s = 0; s < maxnum; ++s) {
      std::vector<WapItem> items;
      for (int f = f0; f < wend; ++f) {
        const int ik = ctx->st[f] + s;
        if (ik > ctx->en[f]) continue;
        float td = (ik - ctx->ft[f]) / ctx->tunit;
        td = mac_min(mac_max(-1.0f, td), 1.0f);
        items.push_back(WapItem{f, ik, td});
      }
      TRY(wap_step(ctx, items, sch->bp_exact));
      for (const WapItem &it : items) TRY(notify(ctx, WAP_EV_WARP, it.frame, it.proj, vol_ptr(ctx, it.frame)));
    }
  return WAP_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
namespace wap {
size_t flow_pairs_bytes(const int vol[3], int flow_scales, float flow_eta) {
  // y: two buffers of 5 pair planes, v: two of 2, u: one of 2 (4 bytes a pair)
  size_t b = 0;
  float t_eta = 1.0f;
  for (int l = 0; l < std::max(flow_scales, 1); ++l) {
    size_t m = 1;
    for (int a = 0; a < 3; ++a) m *= (size_t)std::max(1, (int)(vol[a] * t_eta));
    b += (size_t)4 * (2 * 5 + 2 * 2 + 2) * m;
    t_eta *= flow_eta;
  }
  return b;
}
}  // namespace wap

extern "C" {

int wap_create(wap_ctx **out, const wap_scan_desc *scan, const double *h_angles_deg, int device) try {
  if (!out || !scan || !h_angles_deg) return WAP_EINVAL;
  *out = nullptr;
  for (int a = 0; a < 3; ++a)
    if (scan->vol[a] < 3 || scan->vol[a] > 65535) return WAP_EINVAL;
  if (scan->det[0] < 5 || scan->det[1] < 5 || scan->det[0] > 65535 || scan->det[1] > 65535 || scan->nproj < 1 ||
      scan->nframes_cli < 1)
    return WAP_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return WAP_ENODEV;
  std::unique_ptr<wap_ctx> c(new wap_ctx);
  wap_ctx *ctx = c.get();
  ctx->device = device;
  CU(cudaSetDevice(device));
  CU(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  ctx->own_stream = true;
  ctx->scan = *scan;
  for (int a = 0; a < 3; ++a) ctx->sg.vol[a] = scan->vol[a];
  ctx->sg.det[0] = scan->det[0];
  ctx->sg.det[1] = scan->det[1];
  ctx->sg.vs = scan->vs;
  ctx->sg.ds = scan->ds;
  ctx->sg.sid = scan->sid;
  ctx->sg.sdd = scan->sdd;
  for (int a = 0; a < 3; ++a) ctx->sg.oxyz[a] = scan->oxyz[a];
  ctx->angles.assign(h_angles_deg, h_angles_deg + scan->nproj);
  ctx->h_geom.resize(scan->nproj);
  for (int p = 0; p < scan->nproj; ++p) ctx->h_geom[p] = projection_geometry(ctx->sg, ctx->angles[p]);
  TRY(upload(ctx, ctx->geom, ctx->h_geom));
  ctx->sd = sample_distance(scan->vs);
  ctx->halfW = half_frustum(scan->det[0], scan->ds);
  ctx->halfH = half_frustum(scan->det[1], scan->ds);
  ctx->np = (size_t)scan->det[0] * scan->det[1];
  ctx->nv = (size_t)scan->vol[0] * scan->vol[1] * scan->vol[2];
  CU(ctx->maxbits.ensure(sizeof(unsigned)));
  CU(ctx->zero_vol.ensure(sizeof(float) * 3 * ctx->nv));
  CU(cudaMemsetAsync(ctx->zero_vol.p, 0, sizeof(float) * 3 * ctx->nv, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  *out = c.release();
  return WAP_OK;
} WAP_CATCH

int wap_create_compute(wap_ctx **out, int device) try {
  if (!out) return WAP_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return WAP_ENODEV;
  std::unique_ptr<wap_ctx> c(new wap_ctx);
  wap_ctx *ctx = c.get();
  ctx->device = device;
  CU(cudaSetDevice(device));
  CU(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  ctx->own_stream = true;
  CU(ctx->maxbits.ensure(sizeof(unsigned)));
  *out = c.release();
  return WAP_OK;
} WAP_CATCH

int wap_alloc(wap_ctx *ctx, size_t bytes, void **d_out) try {
  CHECK(ctx && d_out, WAP_EINVAL, "null argument");
  *d_out = nullptr;
  CU(cudaSetDevice(ctx->device));
  cudaError_t e = cudaMalloc(d_out, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *d_out = nullptr;
    return fail(ctx, WAP_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return WAP_OK;
} WAP_CATCH

int wap_free(wap_ctx *ctx, void *d_ptr) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  if (d_ptr) {
    CU(cudaStreamSynchronize(ctx->stream));
    CU(cudaFree(d_ptr));
  }
  return WAP_OK;
} WAP_CATCH

int wap_copy_to_device(wap_ctx *ctx, void *d_dst, const void *h_src, size_t bytes) try {
  CHECK(ctx && (bytes == 0 || (d_dst && h_src)), WAP_EINVAL, "null argument");
  if (bytes) CU(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_copy_to_host(wap_ctx *ctx, void *h_dst, const void *d_src, size_t bytes) try {
  CHECK(ctx && (bytes == 0 || (h_dst && d_src)), WAP_EINVAL, "null argument");
  if (bytes) CU(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_fill_zero(wap_ctx *ctx, void *d_ptr, size_t bytes) try {
  CHECK(ctx && (bytes == 0 || d_ptr), WAP_EINVAL, "null argument");
  if (bytes) CU(cudaMemsetAsync(d_ptr, 0, bytes, ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_set_observer(wap_ctx *ctx, wap_observer_fn fn, void *user) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  ctx->observer = fn;
  ctx->observer_user = user;
  return WAP_OK;
} WAP_CATCH

void wap_destroy(wap_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  const bool idle = !ctx->stream || cudaStreamSynchronize(ctx->stream) == cudaSuccess;
  cudaStream_t s = ctx->own_stream ? ctx->stream : nullptr;
  for (cudaEvent_t e : ctx->pd_events)
    if (e) cudaEventDestroy(e);
  for (wap_ctx *h : ctx->lanes) wap_destroy(h);
  g_recycle = idle;  // the stream has drained: the blocks go to the cache
  delete ctx;
  g_recycle = false;
  if (s) cudaStreamDestroy(s);
}

size_t wap_cached_bytes(void) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  return g_cache_bytes;
}

size_t wap_trim_cache(int device) { return cache_trim(device); }

const char *wap_last_error(const wap_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int wap_set_stream(wap_ctx *ctx, void *cuda_stream) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  if (ctx->own_stream && ctx->stream) {
    CU(cudaStreamSynchronize(ctx->stream));
    cudaStreamDestroy(ctx->stream);
  }
  ctx->stream = (cudaStream_t)cuda_stream;
  ctx->own_stream = false;
  return WAP_OK;
} WAP_CATCH

int wap_synchronize(wap_ctx *ctx) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_get_stats(wap_ctx *ctx, wap_stats *out) try {
  CHECK(ctx && out, WAP_EINVAL, "null argument");
  *out = ctx->stats;
  return WAP_OK;
} WAP_CATCH

int wap_set_profiling(wap_ctx *ctx, int on) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  if (on && ctx->pd_events.empty()) {
    std::vector<cudaEvent_t> ev(2 * 50, nullptr);
    for (auto &e : ev) {
      const cudaError_t r = cudaEventCreate(&e);
      if (r != cudaSuccess) {  // none kept: profiling stays off
        for (cudaEvent_t x : ev)
          if (x) cudaEventDestroy(x);
        return fail(ctx, WAP_ECUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(r));
      }
    }
    ctx->pd_events.swap(ev);
  }
  ctx->profiling = on ? 1 : 0;
  return WAP_OK;
} WAP_CATCH

int wap_set_tuning(wap_ctx *ctx, const char *key, int value) try {
  CHECK(ctx && key, WAP_EINVAL, "null argument");
  const std::string k = key;
  if (k == "pd_form") {
    CHECK(value >= 0 && value <= 3, WAP_EINVAL, "pd_form must be 0, 1, 2 or 3");
    ctx->pd_form = value;
  } else if (k == "flow_bits") {  // each precision keeps its own tuned plans
    CHECK(value == 32 || value == 16, WAP_EINVAL, "flow_bits must be 32 or 16");
    ctx->flow_bits = value;
    return WAP_OK;
  } else if (k == "fp_bricks") {
    CHECK(value == 0 || value == 1, WAP_EINVAL, "fp_bricks must be 0 or 1");
    ctx->fp_bricks = value;
    return WAP_OK;
  } else if (k == "splat_form") {
    CHECK(value == 0 || value == 1, WAP_EINVAL, "splat_form must be 0 or 1");
    ctx->splat_direct = value;
    return WAP_OK;
  } else if (k == "bp_ray") {
    CHECK(value == 0 || value == 1, WAP_EINVAL, "bp_ray must be 0 or 1");
    ctx->bp_ray = value;
    return WAP_OK;
  } else if (k == "flow_lanes") {
    CHECK(value >= 0 && value <= 8, WAP_EINVAL, "flow_lanes must be 0 (automatic) .. 8");
    ctx->flow_lanes = value;
    return WAP_OK;
  } else if (k == "pd_zchunk") {
    CHECK(value >= 0, WAP_EINVAL, "pd_zchunk must be >= 0");
    ctx->pd_zchunk = value;
  } else {
    return fail(ctx, WAP_EINVAL, "unknown tuning key: " + k);
  }
  ctx->pd_plans.clear();
  ctx->pd_plans16.clear();
  return WAP_OK;
} WAP_CATCH

int wap_get_tuning(wap_ctx *ctx, const int *dims, int *h_form, int *h_zchunk) try {
  CHECK(ctx && dims && h_form && h_zchunk, WAP_EINVAL, "null argument");
  const auto &plans = ctx->flow_bits == 16 ? ctx->pd_plans16 : ctx->pd_plans;  // the current precision's plans
  auto it = plans.find(std::make_tuple(dims[0], dims[1], dims[2]));
  *h_form = it == plans.end() ? ctx->pd_form : it->second.first;
  *h_zchunk = it == plans.end() ? ctx->pd_zchunk : it->second.second;
  return WAP_OK;
} WAP_CATCH

int wap_upload_projections(wap_ctx *ctx, const float *h_projs) try {
  CHECK(ctx && h_projs, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  const size_t n = ctx->np * ctx->scan.nproj;
  CU(ctx->projs_own.ensure(sizeof(float) * n));
  CU(cudaMemcpyAsync(ctx->projs_own.p, h_projs, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
  ctx->projs = ctx->projs_own.as<float>();
  // G_Max = max of the first projection image (projslevel[0][0], WaP_Tomo.cpp:347-348).
  float m = h_projs[0];
  for (size_t i = 1; i < ctx->np; ++i) m = h_projs[i] > m ? h_projs[i] : m;
  ctx->gmax = m;
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_set_projections_device(wap_ctx *ctx, const float *d_projs) try {
  CHECK(ctx && d_projs, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  ctx->projs = d_projs;
  KL(launch_max_reduce(d_projs, ctx->np, ctx->maxbits.as<unsigned>(), ctx->stream));
  unsigned bits = 0;
  CU(cudaMemcpyAsync(&bits, ctx->maxbits.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->gmax = decode_max_bits(bits);
  return WAP_OK;
} WAP_CATCH

float wap_gmax(const wap_ctx *ctx) { return ctx ? ctx->gmax : 0.0f; }

int wap_set_gmax(wap_ctx *ctx, float gmax) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  ctx->gmax = gmax;
  return WAP_OK;
} WAP_CATCH

int wap_projection_geometry(const wap_scan_desc *scan, double angle_deg, float *h_p2m, float *h_m2v, float *h_mvv2m,
                            float *h_eye) try {
  if (!scan || !h_p2m || !h_m2v || !h_mvv2m || !h_eye) return WAP_EINVAL;
  ScanGeometry sg{};
  for (int a = 0; a < 3; ++a) sg.vol[a] = scan->vol[a];
  sg.det[0] = scan->det[0];
  sg.det[1] = scan->det[1];
  sg.vs = scan->vs;
  sg.ds = scan->ds;
  sg.sid = scan->sid;
  sg.sdd = scan->sdd;
  for (int a = 0; a < 3; ++a) sg.oxyz[a] = scan->oxyz[a];
  const ProjGeom g = projection_geometry(sg, angle_deg);
  std::memcpy(h_p2m, g.p2m, sizeof(g.p2m));
  std::memcpy(h_m2v, g.m2v, sizeof(g.m2v));
  std::memcpy(h_mvv2m, g.mvv2m, sizeof(g.mvv2m));
  std::memcpy(h_eye, g.eye, sizeof(g.eye));
  return WAP_OK;
} WAP_CATCH

int wap_level_frames(const wap_scan_desc *scan, int level, int *start, int *end, float *ftime, float *tunit, int cap) try {
  if (!scan || level < 0 || level > 4) return -WAP_EINVAL;
  return level_frames(scan->nframes_cli, scan->nproj, level, start, end, ftime, tunit, cap);
} WAP_CATCH

int wap_level_setup(wap_ctx *ctx, int level) try {
  CHECK(ctx, WAP_EINVAL, "null context");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  CHECK(level >= 0 && level <= 4, WAP_EINVAL, "level out of range");
  const int F = level_frames(ctx->scan.nframes_cli, ctx->scan.nproj, level, nullptr, nullptr, nullptr, nullptr, 0);
  ctx->st.assign(F, 0);
  ctx->en.assign(F, 0);
  ctx->ft.assign(F, 0.0f);
  level_frames(ctx->scan.nframes_cli, ctx->scan.nproj, level, ctx->st.data(), ctx->en.data(), ctx->ft.data(),
               &ctx->tunit, F);
  ctx->level = level;
  ctx->F = F;
  ctx->maxwin = 0;
  for (int f = 0; f < F; ++f) ctx->maxwin = std::max(ctx->maxwin, ctx->en[f] - ctx->st[f] + 1);
  const size_t nv = ctx->nv;
  CU(ctx->vols.ensure(sizeof(float) * F * nv));
  CU(ctx->flows.ensure(sizeof(float) * F * 3 * nv));
  CU(ctx->ytv.ensure(sizeof(float) * F * 3 * nv));
  CU(ctx->ytp.ensure(sizeof(float) * F * nv));
  CU(ctx->xbar.ensure(sizeof(float) * F * nv));
  CU(ctx->xprev.ensure(sizeof(float) * F * nv));
  CU(cudaMemsetAsync(ctx->vols.p, 0, sizeof(float) * F * nv, ctx->stream));
  CU(cudaMemsetAsync(ctx->flows.p, 0, sizeof(float) * F * 3 * nv, ctx->stream));
  CU(cudaMemsetAsync(ctx->ytv.p, 0, sizeof(float) * F * 3 * nv, ctx->stream));
  CU(cudaMemsetAsync(ctx->ytp.p, 0, sizeof(float) * F * nv, ctx->stream));
  CU(cudaMemsetAsync(ctx->xbar.p, 0, sizeof(float) * F * nv, ctx->stream));
  CU(cudaMemsetAsync(ctx->xprev.p, 0, sizeof(float) * F * nv, ctx->stream));
  TRY(ensure_level_buffers(ctx));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_level_nframes(const wap_ctx *ctx) { return ctx ? ctx->F : 0; }

int wap_frame_volume_upload(wap_ctx *ctx, int frame, const float *h_vol) try {
  CHECK(ctx && h_vol, WAP_EINVAL, "null argument");
  CHECK(frame >= 0 && frame < ctx->F, WAP_EINVAL, "frame out of range");
  CU(cudaMemcpyAsync(vol_ptr(ctx, frame), h_vol, sizeof(float) * ctx->nv, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_frame_volume_download(wap_ctx *ctx, int frame, float *h_vol) try {
  CHECK(ctx && h_vol, WAP_EINVAL, "null argument");
  CHECK(frame >= 0 && frame < ctx->F, WAP_EINVAL, "frame out of range");
  CU(cudaMemcpyAsync(h_vol, vol_ptr(ctx, frame), sizeof(float) * ctx->nv, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_frame_flow_upload(wap_ctx *ctx, int frame, const float *h_flow) try {
  CHECK(ctx && h_flow, WAP_EINVAL, "null argument");
  CHECK(frame >= 0 && frame < ctx->F, WAP_EINVAL, "frame out of range");
  CU(cudaMemcpyAsync(flow_ptr(ctx, frame), h_flow, sizeof(float) * 3 * ctx->nv, cudaMemcpyHostToDevice,
                     ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_frame_flow_download(wap_ctx *ctx, int frame, float *h_flow) try {
  CHECK(ctx && h_flow, WAP_EINVAL, "null argument");
  CHECK(frame >= 0 && frame < ctx->F, WAP_EINVAL, "frame out of range");
  CU(cudaMemcpyAsync(h_flow, flow_ptr(ctx, frame), sizeof(float) * 3 * ctx->nv, cudaMemcpyDeviceToHost,
                     ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

float *wap_frame_volume_device(wap_ctx *ctx, int frame) {
  if (!ctx || frame < 0 || frame >= ctx->F) return nullptr;
  return vol_ptr(ctx, frame);
}

float *wap_frame_flow_device(wap_ctx *ctx, int frame) {
  if (!ctx || frame < 0 || frame >= ctx->F) return nullptr;
  return flow_ptr(ctx, frame);
}

int wap_level_advance(wap_ctx *ctx) try {
  CHECK(ctx && ctx->level >= 0, WAP_ESTATE, "no level set up");
  const int F0 = ctx->F;
  const size_t nv = ctx->nv;
  DevMem old;
  CU(old.ensure(sizeof(float) * F0 * nv));
  CU(cudaMemcpyAsync(old.p, ctx->vols.p, sizeof(float) * F0 * nv, cudaMemcpyDeviceToDevice, ctx->stream));
  TRY(wap_level_setup(ctx, ctx->level + 1));
  for (int i = 0; i < F0; ++i)
    for (int k = 0; k < 2; ++k)
      if (2 * i + k < ctx->F)
        CU(cudaMemcpyAsync(vol_ptr(ctx, 2 * i + k), old.as<float>() + (size_t)i * nv, sizeof(float) * nv,
                           cudaMemcpyDeviceToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_forward_project(wap_ctx *ctx, int proj, const float *d_vol, float *d_img, float *d_len, float *d_weight) try {
  return wap_forward_project_batch(ctx, 1, &proj, &d_vol, &d_img, &d_len, &d_weight);
} WAP_CATCH

int wap_forward_project_batch(wap_ctx *ctx, int njobs, const int *h_proj, const float *const *h_d_vols,
                              float *const *h_d_imgs, float *const *h_d_lens, float *const *h_d_weights) try {
  CHECK(ctx && h_proj && h_d_vols, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  CHECK(njobs >= 1 && njobs <= 65535, WAP_EINVAL, "job count out of range");
  std::vector<FpJob> jobs(njobs);
  const size_t bf = brick_floats(ctx->scan.vol);
  const bool bricks = ctx->fp_bricks != 0 && brick_room(ctx, bf * njobs);
  for (int q = 0; q < njobs; ++q) {
    CHECK(h_proj[q] >= 0 && h_proj[q] < ctx->scan.nproj, WAP_EINVAL, "projection index out of range");
    CHECK(h_d_vols[q], WAP_EINVAL, "null volume");
    FpJob j{};
    j.vol = h_d_vols[q];
    if (bricks) {  // the projector reads a brick-layout copy
      float *b = ctx->bricks.as<float>() + (size_t)q * bf;
      KL(launch_brick(h_d_vols[q], b, ctx->scan.vol, ctx->stream));
      j.vol = b;
    }
    j.proj = h_proj[q];
    j.img = h_d_imgs ? h_d_imgs[q] : nullptr;
    j.len = h_d_lens ? h_d_lens[q] : nullptr;
    j.weight = h_d_weights ? h_d_weights[q] : nullptr;
    jobs[q] = j;
  }
  TRY(upload(ctx, ctx->jobs_misc, jobs));
  KL(launch_forward(ctx->geom.as<ProjGeom>(), ctx->jobs_misc.as<FpJob>(), njobs, ctx->scan.vol, ctx->scan.det[0],
                    ctx->scan.det[1], ctx->sd, ctx->scan.alpha, ctx->stream, bricks));
  ctx->stats.fp_launches++;
  return WAP_OK;
} WAP_CATCH

int wap_correction(wap_ctx *ctx, int n, const float *d_meas, const float *d_img, const float *d_len, float *d_dual,
                   float *d_corr) try {
  CHECK(ctx && d_meas && d_img && d_len && d_corr, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  KL(launch_correction(n, d_meas, d_img, d_len, d_dual, ctx->scan.alpha, d_corr, ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_backproject_voxel(wap_ctx *ctx, int proj, const float *d_corr, const int *box, int mode, int exact,
                          float *d_vol) try {
  CHECK(ctx && d_corr && box && d_vol, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  CHECK(proj >= 0 && proj < ctx->scan.nproj, WAP_EINVAL, "projection index out of range");
  CHECK(mode == 0 || mode == 1, WAP_EINVAL, "mode must be 0 or 1");
  for (int a = 0; a < 3; ++a)
    CHECK(box[2 * a] >= 0 && box[2 * a + 1] <= ctx->scan.vol[a] && box[2 * a] <= box[2 * a + 1], WAP_EINVAL,
          "box outside the volume");
  BpJob b{};
  b.vol = d_vol;
  b.corr = d_corr;
  b.proj = proj;
  std::memcpy(b.box, box, sizeof(b.box));
  std::vector<BpJob> jobs{b};
  TRY(upload(ctx, ctx->jobs_misc, jobs));
  int mb[3] = {box[1] - box[0], box[3] - box[2], box[5] - box[4]};
  KL(launch_bp_voxel(ctx->geom.as<ProjGeom>(), ctx->jobs_misc.as<BpJob>(), 1, mb, ctx->scan.vol, ctx->scan.det[0],
                     ctx->scan.det[1], ctx->halfW, ctx->halfH, (float)ctx->scan.sdd, ctx->scan.ds, ctx->scan.alpha,
                     ctx->gmax, mode, exact, ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_backproject_ray(wap_ctx *ctx, int proj, const float *d_corr, float *d_contrib, float *d_weight) try {
  CHECK(ctx && d_corr && d_contrib && d_weight, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  CHECK(proj >= 0 && proj < ctx->scan.nproj, WAP_EINVAL, "projection index out of range");
  std::vector<SplatJob> jobs{SplatJob{d_corr, proj, d_contrib, d_weight}};
  TRY(upload(ctx, ctx->jobs_misc, jobs));
  KL(launch_ray_splat(ctx->geom.as<ProjGeom>(), ctx->jobs_misc.as<SplatJob>(), 1, ctx->scan.vol, ctx->scan.det[0],
                      ctx->scan.det[1], ctx->sd, ctx->stream, ctx->splat_direct != 0));
  return WAP_OK;
} WAP_CATCH

int wap_advect(wap_ctx *ctx, const int *dims, const float *aabb, const float *d_vel, const float *d_src, int nc,
               float dt, float *d_out) try {
  CHECK(ctx && dims && aabb && d_vel && d_src && d_out, WAP_EINVAL, "null argument");
  CHECK(dims[0] >= 3 && dims[1] >= 3 && dims[2] >= 3 && nc >= 1, WAP_EINVAL, "grid must be at least 3^3");
  CHECK(aabb[1] > aabb[0] && aabb[3] > aabb[2] && aabb[5] > aabb[4], WAP_EINVAL, "empty bounding box");
  std::vector<float> h(dims[0] + dims[1] + dims[2]);
  world_table(dims, aabb, h.data());
  TRY(upload(ctx, ctx->adv_tab, h));
  std::vector<AdvectJob> jobs{AdvectJob{d_vel, d_src, d_out, dt}};
  TRY(upload(ctx, ctx->jobs_misc, jobs));
  CU(ctx->adv_flags.ensure(sizeof(int) * 2));
  KL(launch_advect(dims, aabb, ctx->adv_tab.as<float>(), ctx->jobs_misc.as<AdvectJob>(), 1, nc, ctx->stream, false,
                   ctx->adv_flags.as<int>()));
  CU(cudaStreamSynchronize(ctx->stream));  // the host table and job list are reused by the next call
  return WAP_OK;
} WAP_CATCH

int wap_blur(wap_ctx *ctx, const int *dims, int nc, float sigma, const float *d_src, float *d_out) try {
  CHECK(ctx && dims && d_src && d_out, WAP_EINVAL, "null argument");
  return do_blur(ctx, dims, nc, sigma, d_src, d_out);
} WAP_CATCH

int wap_resize(wap_ctx *ctx, const int *dims, int nc, const float *d_src, const int *odims, float *d_out) try {
  CHECK(ctx && dims && odims && d_src && d_out, WAP_EINVAL, "null argument");
  for (int a = 0; a < 3; ++a) CHECK(dims[a] >= 1 && odims[a] >= 1, WAP_EINVAL, "empty grid");
  return do_resize(ctx, dims, nc, d_src, odims, d_out);
} WAP_CATCH

int wap_check_packed_cubic(wap_ctx *ctx, unsigned long long n, unsigned long long seed,
                           unsigned long long *h_mismatches) try {
  CHECK(ctx && h_mismatches, WAP_EINVAL, "null argument");
  CU(cudaSetDevice(ctx->device));
  DevMem bad;
  CU(bad.ensure(sizeof(unsigned long long)));
  CU(cudaMemsetAsync(bad.p, 0, sizeof(unsigned long long), ctx->stream));
  KL(launch_cubic_pair_check(n, seed, bad.as<unsigned long long>(), ctx->stream));
  CU(cudaMemcpyAsync(h_mismatches, bad.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_flow_level(wap_ctx *ctx, const int *dims, const float *d_I1, const float *d_I2, float *d_V, float *d_Y1,
                   float *d_Y2, float *d_Y3, float *d_Y4, float tol, float lambda, int max_iters, int nwarps,
                   const float *aabb, const int *roi6, int *h_iters) try {
  CHECK(ctx && dims && d_I1 && d_I2 && d_V && d_Y1 && d_Y2 && d_Y3 && d_Y4 && aabb && roi6, WAP_EINVAL,
        "null argument");
  CHECK(dims[0] >= 3 && dims[1] >= 3 && dims[2] >= 3, WAP_EINVAL, "grid must be at least 3^3");
  float *Y[4] = {d_Y1, d_Y2, d_Y3, d_Y4};
  TRY(flow_level(ctx, dims, d_I1, d_I2, d_V, Y, tol, lambda, max_iters, nwarps, aabb, roi6, h_iters, nullptr));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_flow_multiscale(wap_ctx *ctx, const int *dims, const float *d_I1, const float *d_I2, const float *d_V0,
                        float tol, float lambda, int max_iters, int nwarps, float eta, float sigma, int scales,
                        const int *cut6, float *d_Vout, long long *h_total_iters) try {
  CHECK(ctx && dims && d_I1 && d_I2 && d_V0 && cut6 && d_Vout, WAP_EINVAL, "null argument");
  long long tot = 0;
  TRY(flow_multiscale(ctx, dims, d_I1, d_I2, d_V0, tol, lambda, max_iters, nwarps, eta, sigma, scales, cut6, d_Vout,
                      &tot));
  if (h_total_iters) *h_total_iters = tot;
  return WAP_OK;
} WAP_CATCH

int wap_flow_multiscale_warm(wap_ctx *ctx, const int *dims, const float *d_I1, const float *d_I2, const float *d_V0,
                             const float *d_Y1, const float *d_Y2, const float *d_Y3, const float *d_Y4, float tol,
                             float lambda, int max_iters, int nwarps, float eta, float sigma, int scales,
                             const int *cut6, float *d_Vout, long long *h_total_iters) try {
  CHECK(ctx && dims && d_I1 && d_I2 && d_V0 && cut6 && d_Vout, WAP_EINVAL, "null argument");
  CHECK((d_Y1 && d_Y2 && d_Y3 && d_Y4) || (!d_Y1 && !d_Y2 && !d_Y3 && !d_Y4), WAP_EINVAL,
        "give all four dual fields or none");
  long long tot = 0;
  const float *Y0[4] = {d_Y1, d_Y2, d_Y3, d_Y4};
  TRY(flow_multiscale(ctx, dims, d_I1, d_I2, d_V0, tol, lambda, max_iters, nwarps, eta, sigma, scales, cut6, d_Vout,
                      &tot, d_Y1 ? Y0 : nullptr));
  if (h_total_iters) *h_total_iters = tot;
  return WAP_OK;
} WAP_CATCH

int wap_sart_prox(wap_ctx *ctx, int frame, int nb_sart, int cut, int exact) try {
  CHECK(ctx && ctx->level >= 0, WAP_ESTATE, "no level set up");
  CHECK(ctx->projs, WAP_ESTATE, "no projections uploaded");
  CHECK(frame >= 0 && frame < ctx->F, WAP_EINVAL, "frame out of range");
  int box[6];
  roi_box(ctx, cut, box);
  std::vector<int> frames{frame};
  TRY(sart_frames(ctx, frames, nb_sart, box, exact));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_warp_and_project(wap_ctx *ctx, int frame, int proj, float rtime, int exact) try {
  CHECK(ctx && ctx->level >= 0, WAP_ESTATE, "no level set up");
  CHECK(ctx->projs, WAP_ESTATE, "no projections uploaded");
  CHECK(frame >= 0 && frame < ctx->F, WAP_EINVAL, "frame out of range");
  CHECK(proj >= 0 && proj < ctx->scan.nproj, WAP_EINVAL, "projection index out of range");
  std::vector<WapItem> items{WapItem{frame, proj, rtime}};
  TRY(wap_step(ctx, items, exact));
  CU(cudaStreamSynchronize(ctx->stream));
  return WAP_OK;
} WAP_CATCH

int wap_adaptive_warp(wap_ctx *ctx, int frame, int nb_warp, int cut, int exact) try {
  CHECK(ctx, WAP_EINVAL, "null argument");
  CHECK(has_scan(ctx), WAP_ESTATE, "context has no scan (wap_create_compute)");
  CHECK(ctx->level >= 0, WAP_ESTATE, "no level set up");
  CHECK(ctx->projs, WAP_ESTATE, "no projections uploaded");
  CHECK(frame >= 0 && frame < ctx->F && nb_warp >= 0, WAP_EINVAL, "frame or sweep count out of range");
  CHECK(cut >= 0 && 2 * cut < ctx->scan.vol[0] && 2 * cut < ctx->scan.vol[1] && 2 * cut < ctx->scan.vol[2], WAP_EINVAL,
        "cut must leave a non-empty ROI");
  return adaptive_warp(ctx, frame, nb_warp, cut, exact);
} WAP_CATCH

int wap_outer_iteration_frames(wap_ctx *ctx, const wap_schedule *sch, int f0, int f1, wap_stats *stats) try {
  TRY(check_schedule(ctx, sch, f0, f1));
  ctx->stats = wap_stats{};
  ScopedEvents ev(4);
  CU(ev.create());
  CU(cudaEventRecord(ev[0], ctx->stream));
  // (1) CP prior + SART proximal steps (WaP_Tomo.cpp:563-698)
  for (int icp = 1; icp <= sch->n_cp; ++icp) TRY(cp_pass(ctx, sch, f0, f1, icp));
  CU(cudaEventRecord(ev[1], ctx->stream));
  // (2) flow for each adjacent pair (WaP_Tomo.cpp:732-777)
  TRY(flow_phase(ctx, sch, f0, f1));
  CU(cudaEventRecord(ev[2], ctx->stream));
  // (3) warp-and-project over each visited frame's window (WaP_Tomo.cpp:796-822)
  TRY(wap_pass(ctx, sch, f0, f1));
  CU(cudaEventRecord(ev[3], ctx->stream));
  CU(cudaEventSynchronize(ev[3]));
  float ms[3];
  for (int q = 0; q < 3; ++q) CU(cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]));
  ctx->stats.ms_cp = ms[0];
  ctx->stats.ms_flow = ms[1];
  ctx->stats.ms_wap = ms[2];
  if (stats) *stats = ctx->stats;
  return WAP_OK;
} WAP_CATCH

int wap_outer_iteration_nsteps(const wap_ctx *ctx, const wap_schedule *sch) try {
  if (!ctx || !sch || ctx->level < 0) return -1;
  return sch->n_cp + std::max(ctx->F - 1, 0) + 1;
} WAP_CATCH

int wap_outer_iteration_step(wap_ctx *ctx, const wap_schedule *sch, int step, wap_stats *stats) try {
  TRY(check_schedule(ctx, sch, 0, ctx ? ctx->F : 0));
  const int nflow = std::max(ctx->F - 1, 0);
  CHECK(step >= 0 && step < sch->n_cp + nflow + 1, WAP_EINVAL, "step out of range");
  ctx->stats = wap_stats{};
  ScopedEvents ev(2);
  CU(ev.create());
  const cudaEvent_t e0 = ev[0], e1 = ev[1];
  CU(cudaEventRecord(e0, ctx->stream));
  int phase = 0;
  if (step < sch->n_cp) {
    TRY(cp_pass(ctx, sch, 0, ctx->F, step + 1));
  } else if (step < sch->n_cp + nflow) {
    phase = 1;
    TRY(flow_pair(ctx, sch, step - sch->n_cp));
  } else {
    phase = 2;
    TRY(wap_pass(ctx, sch, 0, ctx->F));
  }
  CU(cudaEventRecord(e1, ctx->stream));
  CU(cudaEventSynchronize(e1));
  float ms = 0.0f;
  CU(cudaEventElapsedTime(&ms, e0, e1));
  (phase == 0 ? ctx->stats.ms_cp : phase == 1 ? ctx->stats.ms_flow : ctx->stats.ms_wap) = ms;
  if (stats) *stats = ctx->stats;
  return WAP_OK;
} WAP_CATCH

size_t wap_ctx_device_bytes(const wap_ctx *ctx) {
  if (!ctx) return 0;
  size_t b = 0;
  for (const DevMem *m : {&ctx->geom, &ctx->projs_own, &ctx->vols, &ctx->flows, &ctx->ytv, &ctx->ytp, &ctx->xbar,
                          &ctx->xprev, &ctx->zero_vol, &ctx->dual, &ctx->corr, &ctx->warped, &ctx->delta, &ctx->back,
                          &ctx->jobs_fp, &ctx->jobs_bp, &ctx->jobs_adv, &ctx->jobs_acc, &ctx->jobs_misc, &ctx->world,
                          &ctx->maxbits, &ctx->blur_a, &ctx->blur_b, &ctx->rs_a, &ctx->rs_b, &ctx->cg_buf,
                          &ctx->pyr_b1, &ctx->pyr_b2, &ctx->adv_tab, &ctx->bricks, &ctx->jobs_fpb})
    b += m->want;
  for (const auto &kv : ctx->flow_work) {
    const FlowWork &w = *kv.second;
    for (const DevMem *m : {&w.va, &w.vb, &w.y, &w.y2, &w.u, &w.kty, &w.kx4prev, &w.warp, &w.acc, &w.err, &w.world,
                            &w.yh[0], &w.yh[1], &w.vh[0], &w.vh[1], &w.uh})
      b += m->want;
  }
  for (const auto &p : ctx->pyramid)
    if (p)
      for (const DevMem *m : {&p->i1, &p->i2, &p->v, &p->y}) b += m->want;
  for (const auto &kv : ctx->resize_tables)
    for (int q = 0; q < 5; ++q) b += kv.second[q].want;
  return b;
}

size_t wap_job_device_bytes(const wap_scan_desc *scan, const wap_schedule *sch) {
  if (!scan || !sch) return 0;
  const size_t nv = (size_t)scan->vol[0] * scan->vol[1] * scan->vol[2];
  const size_t np = (size_t)scan->det[0] * scan->det[1];
  const int F = level_frames(scan->nframes_cli, scan->nproj, 0, nullptr, nullptr, nullptr, nullptr, 0);
  if (F <= 0) return 0;
  std::vector<int> st(F), en(F);
  std::vector<float> ft(F);
  float tu = 0.0f;
  level_frames(scan->nframes_cli, scan->nproj, 0, st.data(), en.data(), ft.data(), &tu, F);
  size_t maxwin = 0;
  for (int f = 0; f < F; ++f) maxwin = std::max(maxwin, (size_t)(en[f] - st[f] + 1));
  size_t floats = 3 * nv                        // zero flow
                  + np * scan->nproj            // projection stack
                  + (size_t)F * 13 * nv         // volumes, flows, CP state, WaP scratch
                  + (size_t)F * np * (1 + maxwin);  // corrections and dual rows
  // flow: per pyramid level 35 floats/voxel of solver state + 15 of pyramid
  // buffers; resize scratch (10 channels, twice) and blur scratch at full size
  float t_eta = 1.0f;
  for (int l = 0; l < std::max(sch->flow_scales, 1); ++l) {
    size_t m = 1;
    for (int a = 0; a < 3; ++a) m *= (size_t)std::max(1, (int)(scan->vol[a] * t_eta));
    floats += 50 * m;
    t_eta *= sch->flow_eta;
  }
  floats += 24 * nv;
  floats += (size_t)F * brick_floats(scan->vol);  // brick copies for the projector, one per frame of a batch
  const size_t tables = (size_t)scan->nproj * sizeof(ProjGeom) + (size_t)4 * 1024 * 1024;  // geometry, job tables
  return floats * sizeof(float) + tables;
}

int wap_outer_iteration(wap_ctx *ctx, const wap_schedule *sch, wap_stats *stats) try {
  CHECK(ctx && ctx->level >= 0, WAP_ESTATE, "no level set up");
  return wap_outer_iteration_frames(ctx, sch, 0, ctx->F, stats);
} WAP_CATCH

}  // extern "C"

// ===========================================================================
// Batched form (wap_batch.h): the scans' SART steps merged into work-queue
// launches, the CP iteration captured as a CUDA graph, flows and warp-and-
// project overlapped on the scans' streams.
// ===========================================================================
#include <thread>

#include "wap/wap_batch.h"

struct wap_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<wap_ctx *> ctxs;
  int fp_shape = -1, bp_shape = -1;  // -1: autotune on the next outer iteration
  DevMem qfp, qbp, qbrick, counter, bricks;
  std::string err;
};

namespace {

int bfail(wap_batch *b, int code, const std::string &msg) {
  if (b) b->err = msg;
  return code;
}
#define BCU(expr)                                                                                    \
  do {                                                                                               \
    cudaError_t _e = (expr);                                                                         \
    if (_e != cudaSuccess) return bfail(b, WAP_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// The merged SART sweep of one CP iteration: per step the brick copies, the
// projections and the backprojections of every frame of every scan whose
// window has that step, each one work-queue launch.
struct BatchPlan {
  std::vector<QFpJob> fp;
  std::vector<QBpJob> bp;
  std::vector<QBrickJob> br;
  std::vector<int> off;  // step s: jobs [off[s], off[s+1]) in fp / bp / br
  std::vector<int> fp_items, bp_items, br_items;
  int nb_sart = 0, exact = 1;
};

// dry: the tuning form of the jobs (projection images into the correction
// slots with no correction or dual update, backprojection into the delta
// volumes), which changes no state of the scans.
int batch_plan(wap_batch *b, const wap_schedule *sch, BatchPlan &P, bool dry) {
  P = BatchPlan();
  P.nb_sart = sch[0].nb_sart;
  P.exact = sch[0].bp_exact;
  int maxnum = 0;
  std::vector<std::vector<std::vector<int>>> orders(b->ctxs.size());
  for (size_t c = 0; c < b->ctxs.size(); ++c) {
    wap_ctx *x = b->ctxs[c];
    orders[c].resize(x->F);
    for (int f = 0; f < x->F; ++f) {
      sart_order(x->st[f], x->en[f], orders[c][f]);
      maxnum = std::max(maxnum, (int)orders[c][f].size());
    }
  }
  size_t max_slot = 0;
  std::vector<size_t> slot_of;  // brick-copy offset (floats) of each job
  for (int s = 0; s < maxnum; ++s) {
    P.off.push_back((int)P.fp.size());
    size_t slot = 0;
    for (size_t c = 0; c < b->ctxs.size(); ++c) {
      wap_ctx *x = b->ctxs[c];
      int box[6];
      roi_box(x, sch[c].cut, box);
      const size_t bf = brick_floats(x->scan.vol);
      for (int f = 0; f < x->F; ++f) {
        if (s >= (int)orders[c][f].size()) continue;
        const int pid = orders[c][f][s];
        QFpJob q{};
        q.job.proj = pid;
        q.job.corr = x->corr.as<float>() + (size_t)f * x->np;
        if (dry) {
          q.job.img = q.job.corr;
        } else {
          q.job.meas = x->projs;
          q.job.dual = x->dual.as<float>() + ((size_t)f * x->maxwin + (pid - x->st[f])) * x->np;
        }
        q.geom = x->geom.as<ProjGeom>();
        for (int a = 0; a < 3; ++a) q.n[a] = x->scan.vol[a];
        q.W = x->scan.det[0];
        q.H = x->scan.det[1];
        q.sd = x->sd;
        q.alpha = x->scan.alpha;
        q.bricked = x->flow_bits == 16 ? 2 : 1;
        QBrickJob r{};
        r.vol = vol_ptr(x, f);
        r.half = x->flow_bits == 16 ? 1 : 0;
        for (int a = 0; a < 3; ++a) r.n[a] = x->scan.vol[a];
        slot_of.push_back(slot);
        slot += bf;
        QBpJob p{};
        p.job.vol = dry ? x->delta.as<float>() + (size_t)f * x->nv : vol_ptr(x, f);
        p.job.corr = q.job.corr;
        p.job.proj = pid;
        std::memcpy(p.job.box, box, sizeof(box));
        p.geom = q.geom;
        p.P = make_bp_params(x->scan.vol, q.W, q.H, x->halfW, x->halfH, (float)x->scan.sdd, x->scan.ds,
                             x->scan.alpha, x->gmax);
        P.fp.push_back(q);
        P.bp.push_back(p);
        P.br.push_back(r);
      }
    }
    max_slot = std::max(max_slot, slot);
  }
  P.off.push_back((int)P.fp.size());
  BCU(b->bricks.ensure(sizeof(float) * std::max<size_t>(max_slot, 1)));
  for (size_t j = 0; j < P.br.size(); ++j) {
    P.br[j].out = b->bricks.as<float>() + slot_of[j];
    P.fp[j].job.vol = P.br[j].out;
  }
  const int nsteps = (int)P.off.size() - 1;
  for (int s = 0; s < nsteps; ++s) {
    const int o = P.off[s], n = P.off[s + 1] - o;
    P.fp_items.push_back(fp_queue_items(P.fp.data() + o, n, std::max(b->fp_shape, 0)));
    P.bp_items.push_back(bp_queue_items(P.bp.data() + o, n, std::max(b->bp_shape, 0)));
    P.br_items.push_back(brick_queue_items(P.br.data() + o, n));
  }
  return WAP_OK;
}

int batch_upload(wap_batch *b, const BatchPlan &P) {
  BCU(b->qfp.ensure(sizeof(QFpJob) * std::max<size_t>(P.fp.size(), 1)));
  BCU(b->qbp.ensure(sizeof(QBpJob) * std::max<size_t>(P.bp.size(), 1)));
  BCU(b->qbrick.ensure(sizeof(QBrickJob) * std::max<size_t>(P.br.size(), 1)));
  BCU(b->counter.ensure(sizeof(int) * 4));
  if (!P.fp.empty()) {
    BCU(cudaMemcpyAsync(b->qfp.p, P.fp.data(), sizeof(QFpJob) * P.fp.size(), cudaMemcpyHostToDevice, b->stream));
    BCU(cudaMemcpyAsync(b->qbp.p, P.bp.data(), sizeof(QBpJob) * P.bp.size(), cudaMemcpyHostToDevice, b->stream));
    BCU(cudaMemcpyAsync(b->qbrick.p, P.br.data(), sizeof(QBrickJob) * P.br.size(), cudaMemcpyHostToDevice,
                        b->stream));
  }
  BCU(cudaStreamSynchronize(b->stream));
  return WAP_OK;
}

// The launches of one step (brick copies, projections, backprojections).
int batch_step(wap_batch *b, const BatchPlan &P, int s, int mode) {
  const int o = P.off[s], n = P.off[s + 1] - o;
  int *ctr = b->counter.as<int>();
  BCU(launch_brick_queue(b->qbrick.as<QBrickJob>() + o, n, P.br_items[s], ctr, b->stream));
  BCU(launch_fp_queue(b->qfp.as<QFpJob>() + o, n, P.fp_items[s], ctr + 1, std::max(b->fp_shape, 0), b->stream));
  BCU(launch_bp_queue(b->qbp.as<QBpJob>() + o, n, P.bp_items[s], ctr + 2, std::max(b->bp_shape, 0), P.exact, mode,
                      b->stream));
  return WAP_OK;
}

// Tile shapes by timing every shape on the batch's largest step, on the dry
// form of its jobs.
int batch_autotune(wap_batch *b, const wap_schedule *sch) {
  if (b->fp_shape >= 0 && b->bp_shape >= 0) return WAP_OK;
  const int keep_fp = b->fp_shape, keep_bp = b->bp_shape;
  BatchPlan P;
  int best_step = 0, pick_fp = 0, pick_bp = 0;
  float best_fp = 1e30f, best_bp = 1e30f;
  ScopedEvents ev(2);
  BCU(ev.create());
  const cudaEvent_t e0 = ev[0], e1 = ev[1];
  int rc = WAP_OK;
  for (int shape = 0; shape < std::max(kFpShapes, kBpShapes) && rc == WAP_OK; ++shape) {
    b->fp_shape = std::min(shape, kFpShapes - 1);
    b->bp_shape = std::min(shape, kBpShapes - 1);
    rc = batch_plan(b, sch, P, true);
    if (rc == WAP_OK) rc = batch_upload(b, P);
    if (rc != WAP_OK || P.fp.empty()) break;
    if (shape == 0)
      for (size_t s = 0; s + 1 < P.off.size(); ++s)
        if (P.off[s + 1] - P.off[s] > P.off[best_step + 1] - P.off[best_step]) best_step = (int)s;
    const int o = P.off[best_step], n = P.off[best_step + 1] - o;
    int *ctr = b->counter.as<int>();
    cudaError_t e = launch_brick_queue(b->qbrick.as<QBrickJob>() + o, n, P.br_items[best_step], ctr, b->stream);
    float ms[2] = {0.0f, 0.0f};
    for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
      auto go = [&]() {
        return kind == 0 ? launch_fp_queue(b->qfp.as<QFpJob>() + o, n, P.fp_items[best_step], ctr + 1, b->fp_shape,
                                           b->stream)
                         : launch_bp_queue(b->qbp.as<QBpJob>() + o, n, P.bp_items[best_step], ctr + 2, b->bp_shape,
                                           P.exact, 1, b->stream);
      };
      e = go();  // warm-up
      if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
      for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = go();
      if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[kind], e0, e1);
    }
    if (e != cudaSuccess) {
      rc = bfail(b, WAP_ECUDA, std::string("batch tuning: ") + cudaGetErrorString(e));
      break;
    }
    if (shape < kFpShapes && ms[0] < best_fp) best_fp = ms[0], pick_fp = shape;
    if (shape < kBpShapes && ms[1] < best_bp) best_bp = ms[1], pick_bp = shape;
  }
  b->fp_shape = keep_fp >= 0 ? keep_fp : pick_fp;
  b->bp_shape = keep_bp >= 0 ? keep_bp : pick_bp;
  return rc;
}

CpArgs batch_cp_args(wap_ctx *ctx, const int box[6]) {
  CpArgs ca;
  for (int a = 0; a < 3; ++a) ca.n[a] = ctx->scan.vol[a];
  std::memcpy(ca.box, box, sizeof(ca.box));
  ca.f0 = 0;
  ca.F = ctx->F;
  ca.Ftot = ctx->F;
  ca.sigma = (float)(.9 / (8.0f * 1.0f));
  ca.tau = 1.0f;
  ca.tv_w = (float)ctx->scan.tv_w;
  ca.tp_w = (float)ctx->scan.tp_w;
  ca.gmax = ctx->gmax;
  return ca;
}

// One CP iteration over every scan (WaP_Tomo.cpp:563-690): per scan the CP
// dual and primal, then the merged SART sweeps, then per scan the SART floor
// and the over-relaxation.  Stream work only, so it can be captured.
int batch_cp_iteration(wap_batch *b, const wap_schedule *sch, const BatchPlan &P) {
  for (size_t c = 0; c < b->ctxs.size(); ++c) {
    wap_ctx *ctx = b->ctxs[c];
    int box[6];
    roi_box(ctx, sch[c].cut, box);
    const CpArgs ca = batch_cp_args(ctx, box);
    BCU(launch_cp_dual(ca, ctx->xbar.as<float>(), ctx->zero_vol.as<float>(), ctx->ytv.as<float>(),
                       ctx->ytp.as<float>(), b->stream));
    BCU(launch_cp_primal(ca, ctx->ytp.as<float>(), ctx->ytv.as<float>(), ctx->vols.as<float>(),
                         ctx->xprev.as<float>(), b->stream));
    BCU(cudaMemsetAsync(ctx->dual.p, 0, sizeof(float) * ctx->F * ctx->maxwin * ctx->np, b->stream));
  }
  const int nsteps = (int)P.off.size() - 1;
  for (int it = 1; it <= P.nb_sart; ++it)
    for (int s = 0; s < nsteps; ++s) TRY(batch_step(b, P, s, 0));
  for (size_t c = 0; c < b->ctxs.size(); ++c) {
    wap_ctx *ctx = b->ctxs[c];
    int box[6];
    roi_box(ctx, sch[c].cut, box);
    const CpArgs ca = batch_cp_args(ctx, box);
    BCU(launch_roi_floor(ctx->nv * ctx->F, ctx->vols.as<float>(), b->stream));
    BCU(launch_cp_overrelax(ca, ctx->vols.as<float>(), ctx->xprev.as<float>(), ctx->xbar.as<float>(), b->stream));
  }
  return WAP_OK;
}

// stream `dst` waits for the work enqueued on `src` so far
cudaError_t stream_follow(cudaStream_t dst, cudaStream_t src) {
  cudaEvent_t ev;
  cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  e = cudaEventRecord(ev, src);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(dst, ev, 0);
  cudaEventDestroy(ev);
  return e;
}

}  // namespace

extern "C" {

int wap_batch_create(wap_batch **out, wap_ctx *const *ctxs, int n) try {
  if (!out || !ctxs || n < 1) return WAP_EINVAL;
  *out = nullptr;
  std::unique_ptr<wap_batch> b(new wap_batch);
  for (int i = 0; i < n; ++i) {
    wap_ctx *x = ctxs[i];
    if (!x || !has_scan(x) || x->level < 0 || !x->projs) return WAP_ESTATE;
    if (x->device != ctxs[0]->device) return WAP_EINVAL;
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == x) return WAP_EINVAL;
    b->ctxs.push_back(x);
  }
  b->device = ctxs[0]->device;
  if (cudaSetDevice(b->device) != cudaSuccess) return WAP_ENODEV;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return WAP_ECUDA;
  *out = b.release();
  return WAP_OK;
} WAP_CATCH

void wap_batch_destroy(wap_batch *b) {
  if (!b) return;
  if (b->stream) {
    cudaStreamSynchronize(b->stream);
    cudaStreamDestroy(b->stream);
  }
  delete b;
}

const char *wap_batch_last_error(const wap_batch *b) { return b ? b->err.c_str() : "null batch"; }

int wap_batch_set_tuning(wap_batch *b, int fp_shape, int bp_shape) try {
  if (!b || fp_shape < -1 || fp_shape >= kFpShapes || bp_shape < -1 || bp_shape >= kBpShapes) return WAP_EINVAL;
  b->fp_shape = fp_shape;
  b->bp_shape = bp_shape;
  return WAP_OK;
} WAP_CATCH

int wap_batch_get_tuning(const wap_batch *b, int *h_fp_shape, int *h_bp_shape) try {
  if (!b || !h_fp_shape || !h_bp_shape) return WAP_EINVAL;
  *h_fp_shape = b->fp_shape;
  *h_bp_shape = b->bp_shape;
  return WAP_OK;
} WAP_CATCH

int wap_batch_outer_iteration(wap_batch *b, const wap_schedule *scheds, wap_stats *stats) try {
  if (!b || !scheds) return WAP_EINVAL;
  const int n = (int)b->ctxs.size();
  for (int c = 0; c < n; ++c) {
    const int rc = check_schedule(b->ctxs[c], &scheds[c], 0, b->ctxs[c]->F);
    if (rc != WAP_OK) return bfail(b, rc, "scan " + std::to_string(c) + ": " + b->ctxs[c]->err);
    if (scheds[c].nb_sart != scheds[0].nb_sart || scheds[c].bp_exact != scheds[0].bp_exact ||
        scheds[c].n_cp != scheds[0].n_cp)
      return bfail(b, WAP_EINVAL, "the scans of a batch share n_cp, nb_sart and bp_exact");
  }
  BCU(cudaSetDevice(b->device));
  for (wap_ctx *x : b->ctxs) {
    x->stats = wap_stats{};
    BCU(stream_follow(b->stream, x->stream));  // the batch follows each scan's earlier work
  }
  ScopedEvents tev(2);
  BCU(tev.create());
  const cudaEvent_t t0 = tev[0], t1 = tev[1];
  BCU(cudaEventRecord(t0, b->stream));
  // (1) CP + SART: tune, plan, capture one CP iteration as a graph, replay it
  warm_queue_kernels();
  TRY(batch_autotune(b, scheds));
  BatchPlan P;
  TRY(batch_plan(b, scheds, P, false));
  TRY(batch_upload(b, P));
  if (scheds[0].n_cp > 0) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = batch_cp_iteration(b, scheds, P);
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
    if (rc != WAP_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    BCU(ec);
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    BCU(ei);
    int rcl = WAP_OK;
    for (int icp = 1; icp <= scheds[0].n_cp && rcl == WAP_OK; ++icp)
      if (cudaGraphLaunch(exec, b->stream) != cudaSuccess) rcl = bfail(b, WAP_ECUDA, "cudaGraphLaunch failed");
    cudaGraphExecDestroy(exec);
    if (rcl != WAP_OK) return rcl;
  }
  // (2) flows and (3) warp-and-project per scan, concurrently on their streams
  std::vector<int> rcs(n, WAP_OK);
  for (wap_ctx *x : b->ctxs) BCU(stream_follow(x->stream, b->stream));
  auto scan_rest = [&](int c) {  // one scan's flows and warp-and-project; exceptions become its status
    try {
      wap_ctx *ctx = b->ctxs[c];
      int rc = cudaSetDevice(b->device) == cudaSuccess ? WAP_OK : WAP_ECUDA;
      for (int f = 0; rc == WAP_OK && f + 1 < ctx->F; ++f) rc = flow_pair(ctx, &scheds[c], f);
      if (rc == WAP_OK) rc = wap_pass(ctx, &scheds[c], 0, ctx->F);
      rcs[c] = rc;
    } catch (const std::bad_alloc &) {
      rcs[c] = WAP_ENOMEM;
    } catch (...) {
      rcs[c] = WAP_EHOST;
    }
  };
  std::vector<std::thread> th;
  int started = 0;
  try {
    th.reserve(n);
    for (; started < n; ++started) th.emplace_back(scan_rest, started);
  } catch (...) {  // no more threads: the remaining scans run here (same results, less overlap)
  }
  for (int c = started; c < n; ++c) scan_rest(c);
  for (auto &t : th) t.join();
  for (int c = 0; c < n; ++c)
    if (rcs[c] != WAP_OK) return bfail(b, rcs[c], "scan " + std::to_string(c) + ": " + b->ctxs[c]->err);
  for (wap_ctx *x : b->ctxs) BCU(stream_follow(b->stream, x->stream));
  BCU(cudaEventRecord(t1, b->stream));
  BCU(cudaEventSynchronize(t1));
  float ms = 0.0f;
  BCU(cudaEventElapsedTime(&ms, t0, t1));
  if (stats) {
    wap_stats s{};
    for (wap_ctx *x : b->ctxs) {
      s.flow_pd_iterations += x->stats.flow_pd_iterations;
      s.kernel_launches += x->stats.kernel_launches;
      s.pd_voxel_iters += x->stats.pd_voxel_iters;
      s.advect_voxels += x->stats.advect_voxels;
      s.projections += x->stats.projections;
      s.backprojections += x->stats.backprojections;
      s.ms_flow += x->stats.ms_flow;
      s.ms_wap += x->stats.ms_wap;
      s.cp_frame_passes += (long long)scheds[0].n_cp * x->F;
    }
    const int nsteps = (int)P.off.size() - 1;
    s.kernel_launches += (long long)scheds[0].n_cp * (3LL * nsteps * P.nb_sart + 4LL * n);
    s.projections += (long long)scheds[0].n_cp * P.nb_sart * (long long)P.fp.size();
    s.backprojections += (long long)scheds[0].n_cp * P.nb_sart * (long long)P.bp.size();
    s.ms_cp = ms;
    *stats = s;
  }
  return WAP_OK;
} WAP_CATCH

}  // extern "C"
