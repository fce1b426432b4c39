// wap19.hpp -- C++ facade with the reference's class and function names
// (WaP19: PSART, VolumeData, TypicalRayProducer, RayCaster,
// SingleScalarVolumePrepare, RayCasterPrepare, GenerateImage_GetCorrections,
// advection::advect, optical_flow::L1TVOpticalFlowNonlinear3D /
// _MultiScale3D, image_cg::cg) over the C ABI in wap.h / wap_io.h.
//
// Header-only; link libwap_gb300.so.  Everything lives in namespace wap19;
// define WAP19_GLOBAL_NAMES before including this header to also get the
// reference's global names (PSART, VolumeData, advection::, ...), so that a
// caller written against the reference's headers compiles unchanged.
//
// Images are host arrays in CImg layout (x fastest, channels planar).  The
// templates accept any image type with width(), height(), depth(),
// spectrum(), data() and an (w, h, d, c) constructor -- CImg<float> is one;
// wap19::Image is a minimal one for callers without CImg.  Failures throw
// wap19::Error (the reference throws CImg exceptions or exits).
#pragma once

#include <algorithm>
#include <cstdio>
#include <cctype>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <sys/stat.h>
#include <type_traits>
#include <vector>

#include "wap/wap.h"
#include "wap/coherent_volume.hpp"
#include "wap/wap_io.h"

namespace wap19 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int st, const wap_ctx *c, const char *what) {
  if (st != WAP_OK) throw Error(st, std::string(what) + " failed (status " + std::to_string(st) + ")" +
                                        (c ? std::string(": ") + wap_last_error(c) : std::string()));
}

// ---- images ----------------------------------------------------------------

class Image {
 public:
  Image() = default;
  Image(int w, int h, int d, int c, float v = 0.0f) : w_(w), h_(h), d_(d), c_(c), v_((size_t)w * h * d * c, v) {}
  int width() const { return w_; }
  int height() const { return h_; }
  int depth() const { return d_; }
  int spectrum() const { return c_; }
  size_t size() const { return v_.size(); }
  bool is_empty() const { return v_.empty(); }
  float *data() { return v_.data(); }
  const float *data() const { return v_.data(); }
  float &operator()(int x, int y, int z, int c = 0) { return v_[x + (size_t)w_ * (y + (size_t)h_ * (z + (size_t)d_ * c))]; }
  float operator()(int x, int y, int z, int c = 0) const {
    return v_[x + (size_t)w_ * (y + (size_t)h_ * (z + (size_t)d_ * c))];
  }
  Image &fill(float v) {
    std::fill(v_.begin(), v_.end(), v);
    return *this;
  }
  Image get_channel(int c) const {
    Image o(w_, h_, d_, 1);
    std::memcpy(o.data(), data() + (size_t)c * w_ * h_ * d_, sizeof(float) * o.size());
    return o;
  }
  // CImg<float>::save_analyze / load_analyze layout (wap_io.h).
  const Image &save_analyze(const char *path) const {
    const int dims[4] = {w_, h_, d_, c_};
    check(wap_analyze_save(path, data(), dims, nullptr), nullptr, "save_analyze");
    return *this;
  }
  static Image load_analyze(const char *path) {
    int dims[4], type = 0;
    check(wap_analyze_info(path, dims, &type), nullptr, "load_analyze");
    Image I(dims[0], dims[1], dims[2], dims[3]);
    check(wap_analyze_load(path, I.data(), I.size()), nullptr, "load_analyze");
    return I;
  }

 private:
  int w_ = 0, h_ = 0, d_ = 0, c_ = 0;
  std::vector<float> v_;
};

template <class image>
inline size_t voxels(const image &I) {
  return (size_t)I.width() * I.height() * I.depth();
}

// ---- device plumbing --------------------------------------------------------

struct CtxDeleter {
  void operator()(wap_ctx *c) const { wap_destroy(c); }
};
using CtxPtr = std::unique_ptr<wap_ctx, CtxDeleter>;

// The calling thread's compute-only context on device 0 (created on first use).
inline wap_ctx *compute_context() {
  thread_local CtxPtr ctx;
  if (!ctx) {
    wap_ctx *c = nullptr;
    check(wap_create_compute(&c, 0), nullptr, "wap_create_compute");
    ctx.reset(c);
  }
  return ctx.get();
}

class DeviceBuffer {
 public:
  DeviceBuffer(wap_ctx *c, size_t nfloats) : c_(c), n_(nfloats) {
    void *p = nullptr;
    check(wap_alloc(c_, sizeof(float) * (n_ ? n_ : 1), &p), c_, "wap_alloc");
    p_ = static_cast<float *>(p);
  }
  ~DeviceBuffer() {
    if (p_) wap_free(c_, p_);
  }
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  float *get() const { return p_; }
  // Copies min(n, size) floats; a NULL or short source leaves zeros behind.
  void upload(const float *h, size_t n) {
    check(wap_fill_zero(c_, p_, sizeof(float) * n_), c_, "wap_fill_zero");
    if (h && n) check(wap_copy_to_device(c_, p_, h, sizeof(float) * std::min(n, n_)), c_, "copy to device");
  }
  void download(float *h, size_t n) const {
    check(wap_copy_to_host(c_, h, p_, sizeof(float) * std::min(n, n_)), c_, "copy to host");
  }

 private:
  wap_ctx *c_;
  size_t n_;
  float *p_ = nullptr;
};

template <class real>
inline void require_float() {
  static_assert(std::is_same<real, float>::value, "the GB300 path computes in float (real = float)");
}

// ---- advection.h ------------------------------------------------------------

namespace advection {
// advection::advect (advection.h:117-146): src warped by vel over dt.  An
// empty vel (a frame whose flow was never computed) is a zero field.
template <typename real, typename image>
image advect(const int *dim, const real *aabb, const image &vel, const image &src, real dt) {
  require_float<real>();
  wap_ctx *c = compute_context();
  const size_t nv = (size_t)dim[0] * dim[1] * dim[2];
  const int nc = src.spectrum();
  DeviceBuffer dv(c, 3 * nv), ds(c, nc * nv), dout(c, nc * nv);
  dv.upload(vel.data(), vel.size());
  ds.upload(src.data(), src.size());
  const float ab[6] = {(float)aabb[0], (float)aabb[1], (float)aabb[2], (float)aabb[3], (float)aabb[4], (float)aabb[5]};
  check(wap_advect(c, dim, ab, dv.get(), ds.get(), nc, (float)dt, dout.get()), c, "advection::advect");
  image out(dim[0], dim[1], dim[2], nc);
  dout.download(out.data(), (size_t)nc * nv);
  return out;
}
}  // namespace advection

// ---- optical_flow.h -----------------------------------------------------------

namespace optical_flow {
inline void require_l1(int norm) {
  if (norm != 1) throw Error(WAP_EINVAL, "optical_flow: only the L1 data term (norm 1, as PSART uses) is provided");
}

// One pyramid level (optical_flow.h:88-995): V and Y1..Y4 updated in place.
template <typename real, typename image>
void L1TVOpticalFlowNonlinear3D(int *dim, const image &image1, const image &image2, image &_inputV, image &_inputY1,
                                image &_inputY2, image &_inputY3, image &_inputY4, float _tol, float _lambda,
                                int _maxIterations, int _norm, int _numberOfWarps, real *_aabb, float huber,
                                int *m_roi) {
  require_float<real>();
  require_l1(_norm);
  (void)huber;  // used only by the Huber data term (norm 4)
  wap_ctx *c = compute_context();
  const size_t nv = (size_t)dim[0] * dim[1] * dim[2];
  DeviceBuffer i1(c, nv), i2(c, nv), v(c, 3 * nv), y1(c, 3 * nv), y2(c, 3 * nv), y3(c, 3 * nv), y4(c, nv);
  i1.upload(image1.data(), nv);
  i2.upload(image2.data(), nv);
  v.upload(_inputV.data(), _inputV.size());
  y1.upload(_inputY1.data(), _inputY1.size());
  y2.upload(_inputY2.data(), _inputY2.size());
  y3.upload(_inputY3.data(), _inputY3.size());
  y4.upload(_inputY4.data(), _inputY4.size());
  const float ab[6] = {(float)_aabb[0], (float)_aabb[1], (float)_aabb[2],
                       (float)_aabb[3], (float)_aabb[4], (float)_aabb[5]};
  std::vector<int> its(_numberOfWarps > 0 ? _numberOfWarps : 1);
  check(wap_flow_level(c, dim, i1.get(), i2.get(), v.get(), y1.get(), y2.get(), y3.get(), y4.get(), _tol, _lambda,
                       _maxIterations, _numberOfWarps, ab, m_roi, its.data()),
        c, "optical_flow::L1TVOpticalFlowNonlinear3D");
  auto fetch = [&](image &dst, const DeviceBuffer &b, int ch) {
    if (voxels(dst) != nv || dst.spectrum() != ch) dst = image(dim[0], dim[1], dim[2], ch);
    b.download(dst.data(), (size_t)ch * nv);
  };
  fetch(_inputV, v, 3);
  fetch(_inputY1, y1, 3);
  fetch(_inputY2, y2, 3);
  fetch(_inputY3, y3, 3);
  fetch(_inputY4, y4, 1);
}

// Coarse-to-fine wrapper (optical_flow.h:1002-1126): returns the finest flow;
// like the reference, the arguments V and Y1..Y4 are read, not updated.
template <typename real, typename image>
image L1TVOpticalFlowNonlinear_MultiScale3D(int *dim, const image &image1, const image &image2, image &_inputV,
                                            image &_inputY1, image &_inputY2, image &_inputY3, image &_inputY4,
                                            real _tol, real _lambda, int _maxIterations, int _norm,
                                            int _numberOfWarps, real eta, real sigma, int scales, real _huber,
                                            int *cut) {
  require_float<real>();
  require_l1(_norm);
  (void)_huber;
  wap_ctx *c = compute_context();
  const size_t nv = (size_t)dim[0] * dim[1] * dim[2];
  DeviceBuffer i1(c, nv), i2(c, nv), v0(c, 3 * nv), out(c, 3 * nv);
  DeviceBuffer y1(c, 3 * nv), y2(c, 3 * nv), y3(c, 3 * nv), y4(c, nv);
  i1.upload(image1.data(), nv);
  i2.upload(image2.data(), nv);
  v0.upload(_inputV.data(), _inputV.size());
  y1.upload(_inputY1.data(), _inputY1.size());
  y2.upload(_inputY2.data(), _inputY2.size());
  y3.upload(_inputY3.data(), _inputY3.size());
  y4.upload(_inputY4.data(), _inputY4.size());
  long long total = 0;
  check(wap_flow_multiscale_warm(c, dim, i1.get(), i2.get(), v0.get(), y1.get(), y2.get(), y3.get(), y4.get(),
                                 (float)_tol, (float)_lambda, _maxIterations, _numberOfWarps, (float)eta,
                                 (float)sigma, scales, cut, out.get(), &total),
        c, "optical_flow::L1TVOpticalFlowNonlinear_MultiScale3D");
  image r(dim[0], dim[1], dim[2], 3);
  out.download(r.data(), 3 * nv);
  return r;
}
}  // namespace optical_flow

// ---- cg.h -------------------------------------------------------------------

namespace image_cg {
// The operator the library provides: A = a*I - b*Laplacian with clamped
// (Neumann) neighbours.  mode 1 reproduces the reference's update
// (image_blas.h:135-149), mode 0 is textbook CG.
struct ScreenedLaplacian {
  float a = 1.0f, b = 1.0f;
  int mode = 1;
};

template <typename real, typename image, typename linear_op>
void cg(linear_op &A, image &x, const image &b, const real rel_tol = 1e-6, const int max_iters = 500,
        const real abs_tol = 1e-9) {
  require_float<real>();
  static_assert(std::is_same<linear_op, ScreenedLaplacian>::value,
                "image_cg::cg on the GPU takes wap19::image_cg::ScreenedLaplacian");
  wap_ctx *c = compute_context();
  const int dims[3] = {b.width(), b.height(), b.depth()};
  const size_t n = b.size();
  DeviceBuffer dx(c, n), db(c, n);
  dx.upload(x.data(), x.size());
  db.upload(b.data(), n);
  int its = 0;
  check(wap_cg_screened_laplacian(c, dims, A.a, A.b, db.get(), dx.get(), (float)rel_tol, max_iters, (float)abs_tol,
                                  A.mode, &its),
        c, "image_cg::cg");
  if (x.size() != n) x = image(dims[0], dims[1], dims[2], b.spectrum());
  dx.download(x.data(), n);
}
}  // namespace image_cg

// ---- VolumeData / Frames -------------------------------------------------------

// Frame_item (Frames.h:16-60): a key frame of a time level.
struct Frame_item {
  float fTime = 0.0f;
  Image fVolume;
  Image fFlow;  // empty until the flow of the frame's pair is computed
  int fprojRange = 0;
  int fStartproj = -1;
  int fEndproj = -1;
};

// VolumeData (VolumeData.cpp:118-228): volume size, spacing and the frame
// lists of the two time levels.
class VolumeData {
 public:
  void setParas(int *vols, double vs, int nframes, int totalproj) {
    for (int a = 0; a < 3; ++a) m_Dims[a] = vols[a];
    m_vs = vs;
    m_nframes = nframes;
    m_totalProjs = totalproj;
  }
  // Frame windows of both levels and zero volumes (VolumeData.cpp:118-228).
  void ReadStructuredFile(int nlevels = 2) {
    wap_scan_desc sd{};
    for (int a = 0; a < 3; ++a) sd.vol[a] = m_Dims[a];
    sd.det[0] = sd.det[1] = 8;
    sd.nproj = m_totalProjs;
    sd.nframes_cli = m_nframes;
    m_Frameslist.assign(nlevels, {});
    m_fInLevel.assign(nlevels, 0);
    m_tUnitInLevel.assign(nlevels, 0.0f);
    for (int l = 0; l < nlevels; ++l) {
      const int F = wap_level_frames(&sd, l, nullptr, nullptr, nullptr, nullptr, 0);
      if (F <= 0) throw Error(WAP_EINVAL, "VolumeData: no frames");
      std::vector<int> st(F), en(F);
      std::vector<float> ft(F);
      float tu = 0.0f;
      wap_level_frames(&sd, l, st.data(), en.data(), ft.data(), &tu, F);
      m_fInLevel[l] = F;
      m_tUnitInLevel[l] = tu;
      for (int f = 0; f < F; ++f) {
        Frame_item it;
        it.fTime = ft[f];
        it.fStartproj = st[f];
        it.fEndproj = en[f];
        it.fprojRange = en[f] - st[f];
        it.fVolume = Image(m_Dims[0], m_Dims[1], m_Dims[2], 1, 0.0f);
        m_Frameslist[l].push_back(std::move(it));
      }
    }
  }
  void GetDimensions(int *dims) const {
    for (int a = 0; a < 3; ++a) dims[a] = m_Dims[a];
  }
  void GetSpacings(float *sp) const {
    for (int a = 0; a < 3; ++a) sp[a] = (float)m_vs;
  }
  int m_Dims[3] = {0, 0, 0};
  double m_vs = 1.0;
  int m_nframes = 1;
  int m_totalProjs = 0;
  std::vector<std::vector<Frame_item>> m_Frameslist;
  std::vector<int> m_fInLevel;
  std::vector<float> m_tUnitInLevel;
};

// ---- projector entry points ------------------------------------------------------

class PSART;

// TypicalRayProducer (TypicalRayProducer.cpp:40-105): owns the W*H outputs of
// one projection.  PSART binds it to its context.
class TypicalRayProducer {
 public:
  TypicalRayProducer(int vx, int vy, int vz, int W, int H, double ds, const char *bp = "Voxelbased")
      : m_W(W), m_H(H), m_ds(ds), m_bp(bp ? bp : "Voxelbased"),
        m_Image((size_t)W * H), m_Length((size_t)W * H), m_Weight((size_t)W * H), m_Corr((size_t)W * H) {
    m_Vol[0] = vx;
    m_Vol[1] = vy;
    m_Vol[2] = vz;
    m_ImageData = m_Image.data();
    m_imageraylength = m_Length.data();
    m_WeightOfImage = m_Weight.data();
    m_Correction = m_Corr.data();
  }
  float *GetContributions() { return nullptr; }
  float *GetTotalWeight() { return nullptr; }
  float *GetCorrection() { return m_Correction; }
  // Public like the reference's: projection, ray length, sample count.
  float *m_ImageData, *m_imageraylength, *m_WeightOfImage, *m_Correction;
  int m_W, m_H, m_Vol[3];
  double m_ds;
  std::string m_bp;
  // set by SingleScalarVolumePrepare
  wap_ctx *m_ctx = nullptr;
  int m_proj = -1;
  std::shared_ptr<DeviceBuffer> m_vol;  // the (warped) frame volume on the device

 private:
  std::vector<float> m_Image, m_Length, m_Weight, m_Corr;
};

// RayCaster (RayCaster.cpp): the sample distance comes from the voxel spacing.
class RayCaster {};

inline bool RayCasterPrepare(RayCaster *rc, int size[]) {
  (void)size;
  return rc != nullptr;
}

// ---- PSART --------------------------------------------------------------------------

// PSART (WaP_Tomo.h:20-120, WaP_Tomo.cpp:228-877) on the GPU library.
class PSART {
 public:
  // WaP_Tomo.cpp:228-353.  d1 = TV weight (-s), d2 = temporal weight (-t),
  // d3 (-l) is unused, as in the reference.  Angles are read from
  // angle_file (the reference's fixed "ours_foam_compress.txt"), projections
  // from projsfile[0] split along z into projno images.
  PSART(double d1, double d2, double d3, const char *outputfile, int *imgwh, int projno, int iters, int sartiters,
        double alp, double sid, const char **projsfile, double *oxyz, double sdd, double ds, const char *_prior,
        const char *_bp, int *volxyz, int nframes, double *startdg, int nrounds,
        const char *angle_file = "ours_foam_compress.txt")
      : m_RayProducer(new TypicalRayProducer(volxyz[0], volxyz[1], volxyz[2], imgwh[0], imgwh[1], ds, _bp)) {
    (void)d3;
    (void)iters;
    (void)_prior;
    (void)startdg;
    (void)nrounds;
    m_out = outputfile ? outputfile : "Test/test";
    m_sd.det[0] = imgwh[0];
    m_sd.det[1] = imgwh[1];
    for (int a = 0; a < 3; ++a) m_sd.vol[a] = volxyz[a];
    m_sd.nproj = projno;
    m_sd.nframes_cli = nframes;
    m_sd.ds = ds;
    m_sd.sid = sid;
    m_sd.sdd = sdd;
    for (int a = 0; a < 3; ++a) m_sd.oxyz[a] = oxyz[a];
    m_sd.alpha = alp;
    m_sd.tv_w = d1;
    m_sd.tp_w = d2;
    (void)sartiters;  // Render's own nb_proxiSART = 2 is what the live path uses (WaP_Tomo.cpp:484)
    m_angles.assign(projno, 0.0);
    int got = 0;
    if (wap_read_angles(angle_file, m_angles.data(), projno, &got) != WAP_OK)
      std::fprintf(stderr, "PSART: angle file %s not found; all angles are 0 (as the reference)\n", angle_file);
    else if (got < projno)
      std::fprintf(stderr, "PSART: %s holds %d of %d angles; the rest are 0 (as the reference)\n", angle_file, got,
                   projno);
    if (projsfile && projsfile[0]) load_projections(projsfile[0]);
  }
  ~PSART() { delete m_RayProducer; }
  PSART(const PSART &) = delete;
  PSART &operator=(const PSART &) = delete;

  // WaP_Tomo.cpp:361-434: the context is made here, once the voxel spacing
  // is known.
  void SetData(VolumeData *data) {
    m_Data = data;
    m_sd.vs = data->m_vs;
    wap_ctx *c = nullptr;
    check(wap_create(&c, &m_sd, m_angles.data(), 0), nullptr, "wap_create");
    m_ctx.reset(c);
    if (!m_projs.empty()) {
      check(wap_upload_projections(c, m_projs.data()), c, "wap_upload_projections");
      check(wap_set_gmax(c, m_gmax), c, "wap_set_gmax");
    }
    m_RayProducer->m_ctx = c;
    m_level = -1;
    check(wap_set_tuning(c, "flow_bits", m_flow_bits), c, "flow precision");
    // --bp Raybased: SART backprojects through the matched ray-driven splat
    // with column-sum normalisation (the reference only allocates its sums
    // for this mode, TypicalRayProducer.cpp:42-45,100-104)
    check(wap_set_tuning(c, "bp_ray", m_RayProducer->m_bp == "Raybased" ? 1 : 0), c, "backprojection mode");
  }

  // The whole reconstruction (WaP_Tomo.cpp:473-875); the reference ends the
  // process here (exit(0)), this returns.
  void Render() {
    need_ctx();
    const int nlevels = (int)m_outloop_per_level.size() < m_nlevels ? (int)m_outloop_per_level.size() : m_nlevels;
    for (int lvl = 0; lvl < nlevels; ++lvl) {
      if (lvl == 0) enter_level(0, true);
      else {
        check(wap_level_advance(m_ctx.get()), m_ctx.get(), "wap_level_advance");
        m_level = lvl;
      }
      wap_schedule sc = schedule(lvl);
      for (int outloop = 0; outloop < m_outloop_per_level[lvl]; ++outloop) {
        m_outloop = outloop;
        check(wap_set_observer(m_ctx.get(), m_dump ? &PSART::observe : nullptr, this), m_ctx.get(), "observer");
        check(wap_outer_iteration(m_ctx.get(), &sc, &m_stats), m_ctx.get(), "PSART::Render outer iteration");
        check(wap_set_observer(m_ctx.get(), nullptr, nullptr), m_ctx.get(), "observer");
      }
      sync_frames_to_host(lvl);
    }
  }

  // WaP_Tomo.cpp:1424-1678 on frame `iframes` of level `flevel`.
  void SART_Proximal_Operator(int iframes, int nb_sart, int outloop, int stIter, int flevel) {
    (void)outloop;
    (void)stIter;
    enter_level(flevel, false);
    upload_frame(flevel, iframes);
    check(wap_sart_prox(m_ctx.get(), iframes, nb_sart, m_cut, m_bp_exact), m_ctx.get(), "SART_Proximal_Operator");
    download_frame(flevel, iframes);
  }

  // WaP_Tomo.cpp:1207-1421 for projection iproj of frame iframes.
  void WarpAndProjct(int iproj, int iframes, int *dimension, float rtime, float *aabb, int outloop, int warpiter,
                     char *_file_header, int flevel) {
    (void)dimension;
    (void)aabb;
    (void)outloop;
    (void)warpiter;
    (void)_file_header;
    enter_level(flevel, false);
    const int F = (int)m_Data->m_Frameslist[flevel].size();
    for (int f : {iframes - 1, iframes, iframes + 1})
      if (f >= 0 && f < F) upload_frame(flevel, f);
    check(wap_warp_and_project(m_ctx.get(), iframes, iproj, rtime, m_bp_exact), m_ctx.get(), "WarpAndProjct");
    download_frame(flevel, iframes);
  }

  // ---- settings with the reference's hard-coded defaults (WaP_Tomo.cpp:478-492, 711-727)
  std::vector<int> m_outloop_per_level{1, 1, 1, 1, 1};
  std::vector<int> m_nb_volOpt{2, 10, 21, 6, 21, 15};
  int m_nlevels = 2;
  int m_nb_proxiSART = 2;
  int m_nb_projwarp = 1;
  int m_cut = 8;
  int m_bp_exact = 1;     // 1: the reference's double arithmetic in the bicubic backprojection
  int m_flow_scales = 5;
  int m_flow_iters = 3000;
  float m_flow_tol = 0.008f;
  int m_flow_bits = 32;   // 16: the precision form (FP16 flow-solver state); set before SetData
  bool m_dump = true;     // write the reference's Analyze dumps (SART, flow, warped, WaP)
  std::string m_out;
  wap_stats m_stats{};

  TypicalRayProducer *m_RayProducer;
  VolumeData *m_Data = nullptr;
  wap_ctx *context() const { return m_ctx.get(); }
  const std::vector<double> &angles() const { return m_angles; }
  float gmax() const { return m_gmax; }

 private:
  void need_ctx() const {
    if (!m_ctx) throw Error(WAP_ESTATE, "PSART: SetData has not been called");
  }

  wap_schedule schedule(int lvl) const {
    wap_schedule sc{};
    sc.n_cp = m_nb_volOpt[lvl < (int)m_nb_volOpt.size() ? lvl : (int)m_nb_volOpt.size() - 1];
    sc.nb_sart = m_nb_proxiSART;
    sc.nb_projwarp = m_nb_projwarp;
    sc.wp_frames = m_sd.nframes_cli;  // WaP_Tomo.cpp:801 visits the command line's frame count
    sc.flow_tol = m_flow_tol;
    sc.flow_lambda = 0.05f;
    sc.flow_iters = m_flow_iters;
    sc.flow_warps = 3;
    sc.flow_eta = 0.5f;
    sc.flow_sigma = 0.8f;
    sc.flow_scales = m_flow_scales;
    sc.cut = m_cut;
    sc.bp_exact = m_bp_exact;
    return sc;
  }

  // CImg's load dispatches on the extension (CImg.h:46142-46290): .tif/.tiff
  // through libtiff, Analyze/NIfTI otherwise.
  static bool is_tiff(const char *path) {
    const std::string p(path);
    const size_t dot = p.rfind('.');
    std::string ext = dot == std::string::npos ? "" : p.substr(dot + 1);
    for (char &c : ext) c = (char)std::tolower((unsigned char)c);
    return ext == "tif" || ext == "tiff";
  }

  void load_projections(const char *path) {
    int dims[4], type = 0;
    const bool tiff = is_tiff(path);
    check(tiff ? wap_tiff_info(path, dims, nullptr, nullptr) : wap_analyze_info(path, dims, &type), nullptr,
          "PSART: projection stack");
    const int W = dims[0], H = dims[1], D = dims[2];
    if (W != m_sd.det[0] || H != m_sd.det[1])
      throw Error(WAP_EINVAL, "PSART: projection images are " + std::to_string(W) + "x" + std::to_string(H) +
                                  ", the command line says " + std::to_string(m_sd.det[0]) + "x" +
                                  std::to_string(m_sd.det[1]));
    std::vector<float> stack((size_t)W * H * D * dims[3]);
    check(tiff ? wap_tiff_load(path, stack.data(), stack.size()) : wap_analyze_load(path, stack.data(), stack.size()),
          nullptr, "PSART: projection stack");
    const int P = m_sd.nproj;
    std::vector<int> first(P), count(P);
    check(wap_split_z(D, P, first.data(), count.data()), nullptr, "PSART: split of the projection stack");
    const size_t np = (size_t)W * H;
    m_projs.resize(np * P);
    for (int k = 0; k < P; ++k) std::memcpy(&m_projs[np * k], &stack[np * first[k]], sizeof(float) * np);
    // G_Max = max over the first piece (all of its slices; WaP_Tomo.cpp:347-348)
    float m = stack[0];
    for (size_t i = 0; i < np * count[0]; ++i) m = stack[i] > m ? stack[i] : m;
    m_gmax = m;
  }

  void enter_level(int lvl, bool upload) {
    need_ctx();
    if (m_level == lvl) return;
    check(wap_level_setup(m_ctx.get(), lvl), m_ctx.get(), "wap_level_setup");
    m_level = lvl;
    if (upload)
      for (int f = 0; f < (int)m_Data->m_Frameslist[lvl].size(); ++f) upload_frame(lvl, f);
  }

  void upload_frame(int lvl, int f) {
    const Frame_item &it = m_Data->m_Frameslist[lvl][f];
    if (!it.fVolume.is_empty())
      check(wap_frame_volume_upload(m_ctx.get(), f, it.fVolume.data()), m_ctx.get(), "frame upload");
    if (!it.fFlow.is_empty())
      check(wap_frame_flow_upload(m_ctx.get(), f, it.fFlow.data()), m_ctx.get(), "flow upload");
  }

  void download_frame(int lvl, int f) {
    Frame_item &it = m_Data->m_Frameslist[lvl][f];
    const int *d = m_sd.vol;
    if (it.fVolume.size() != (size_t)d[0] * d[1] * d[2]) it.fVolume = Image(d[0], d[1], d[2], 1);
    check(wap_frame_volume_download(m_ctx.get(), f, it.fVolume.data()), m_ctx.get(), "frame download");
  }

  void sync_frames_to_host(int lvl) {
    const int *d = m_sd.vol;
    for (int f = 0; f < (int)m_Data->m_Frameslist[lvl].size(); ++f) {
      download_frame(lvl, f);
      Frame_item &it = m_Data->m_Frameslist[lvl][f];
      if (it.fFlow.size() != 3 * (size_t)d[0] * d[1] * d[2]) it.fFlow = Image(d[0], d[1], d[2], 3);
      check(wap_frame_flow_download(m_ctx.get(), f, it.fFlow.data()), m_ctx.get(), "flow download");
    }
  }

  static void mkdir_p(const std::string &dir) {
    if (!dir.empty()) ::mkdir(dir.c_str(), 0755);
  }

  // The reference's Analyze dumps, at the points it writes them.
  static void observe(void *user, int event, int level, int a, int b, const float *d_data) {
    PSART *self = static_cast<PSART *>(user);
    wap_ctx *c = self->m_ctx.get();
    const int *d = self->m_sd.vol;
    const size_t nv = (size_t)d[0] * d[1] * d[2];
    char name[1024];
    if (event == WAP_EV_SART) {  // WaP_Tomo.cpp:1669
      const size_t slash = self->m_out.rfind('/');
      if (slash != std::string::npos) mkdir_p(self->m_out.substr(0, slash));
      Image v(d[0], d[1], d[2], 1);
      if (wap_copy_to_host(c, v.data(), d_data, sizeof(float) * nv) != WAP_OK) return;
      std::snprintf(name, sizeof(name), "%s.f%03d.out%02d.st%02d.flevel%02d.hdr", self->m_out.c_str(), a,
                    self->m_outloop, b, level);
      v.save_analyze(name);
    } else if (event == WAP_EV_FLOW) {  // WaP_Tomo.cpp:764-771
      const float smoothness = 0.05f, huber = 1.0f;
      Image fl(d[0], d[1], d[2], 3);
      if (wap_copy_to_host(c, fl.data(), d_data, sizeof(float) * 3 * nv) != WAP_OK) return;
      self->save_warped(a, d_data);
      mkdir_p("VelocityField");
      const char comp[3] = {'u', 'v', 'w'};
      for (int ch = 0; ch < 3; ++ch) {
        std::snprintf(name, sizeof(name), "%s/Flow%03d.s%2.3f.h%1.3f.f%03d.outloop%03d.%c.hdr", "VelocityField",
                      d[0], smoothness, huber, a, self->m_outloop, comp[ch]);
        fl.get_channel(ch).save_analyze(name);
      }
    } else if (event == WAP_EV_WARP) {  // WaP_Tomo.cpp:1417-1418 (warpiter 0)
      Image v(d[0], d[1], d[2], 1);
      if (wap_copy_to_host(c, v.data(), d_data, sizeof(float) * nv) != WAP_OK) return;
      mkdir_p("WarpStep");
      std::snprintf(name, sizeof(name), "%s/f%03d.p%03d.warp%03d.out%02d.flevel%02d.hdr", "WarpStep", a, b, 0,
                    self->m_outloop, level);
      v.save_analyze(name);
    }
  }

  // warpedI dumps after each flow (WaP_Tomo.cpp:762-767): I2 advected by -dt
  // and I1 by +dt with the new flow, dt = 1.
  void save_warped(int f, const float *d_flow) {
    wap_ctx *c = m_ctx.get();
    const int *d = m_sd.vol;
    const size_t nv = (size_t)d[0] * d[1] * d[2];
    const float aabb[6] = {0, (float)d[0], 0, (float)d[1], 0, (float)d[2]};
    DeviceBuffer w(c, nv);
    Image v(d[0], d[1], d[2], 1);
    const float smoothness = 0.05f, huber = 1.0f;
    char name[1024];
    mkdir_p("warpedVolume");
    const float *I1 = wap_frame_volume_device(c, f), *I2 = wap_frame_volume_device(c, f + 1);
    if (wap_advect(c, d, aabb, d_flow, I2, 1, -1.0f, w.get()) == WAP_OK) {
      w.download(v.data(), nv);
      std::snprintf(name, sizeof(name), "warpedVolume/warpedI%03d.s%1.3f.h%3.3f.f%03d.outloop%03d.f%03d_back.hdr", f,
                    smoothness, huber, f, m_outloop, f);
      v.save_analyze(name);
    }
    if (wap_advect(c, d, aabb, d_flow, I1, 1, 1.0f, w.get()) == WAP_OK) {
      w.download(v.data(), nv);
      std::snprintf(name, sizeof(name),
                    "warpedVolume/warpedI%03d.s%1.3f.h%3.3f.f%03d.outloop%03d.f%03d_forward.hdr", f + 1,
                    smoothness, huber, f, m_outloop, f);
      v.save_analyze(name);
    }
  }

  wap_scan_desc m_sd{};
  std::vector<double> m_angles;
  std::vector<float> m_projs;
  float m_gmax = 0.0f;
  CtxPtr m_ctx;
  int m_level = -1;
  int m_outloop = 0;
};

// SingleScalarVolumePrepare (SingleScalarVolume.core.h:366-405): selects the
// frame volume for the next projection, warped to rtime by the frame's flow
// when isWarpped.  Here it also binds the projection id (the reference's
// PSART::RotateVolume before it).
inline bool SingleScalarVolumePrepare(VolumeData *volume, TypicalRayProducer *rp, int frame, bool isWarpped,
                                      int ProjId, float rtime, int flevel) {
  if (!volume || !rp || !rp->m_ctx) return false;
  wap_ctx *c = rp->m_ctx;
  const int *d = volume->m_Dims;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  auto &frames = volume->m_Frameslist[flevel];
  rp->m_vol = std::make_shared<DeviceBuffer>(c, nv);
  rp->m_vol->upload(frames[frame].fVolume.data(), frames[frame].fVolume.size());
  if (isWarpped) {
    const int nf = (int)frames.size() + 2;  // the reference's list carries two padding copies
    const int ff = rtime < 0.0f ? (frame - 1 > 0 ? frame - 1 : 0) : (frame < nf - 1 ? frame : nf - 1);
    DeviceBuffer vel(c, 3 * nv), out(c, nv);
    if (ff < (int)frames.size()) vel.upload(frames[ff].fFlow.data(), frames[ff].fFlow.size());
    else vel.upload(nullptr, 0);
    const float aabb[6] = {0, (float)d[0], 0, (float)d[1], 0, (float)d[2]};
    check(wap_advect(c, d, aabb, vel.get(), rp->m_vol->get(), 1, rtime, out.get()), c, "SingleScalarVolumePrepare");
    std::vector<float> h(nv);
    out.download(h.data(), nv);
    rp->m_vol->upload(h.data(), nv);
  }
  rp->m_proj = ProjId;
  return true;
}

// GenerateImage_GetCorrections (TypicalRayProducer.core.h:230-268): the
// projection, ray length and sample count into the producer's arrays.
inline void GenerateImage_GetCorrections(TypicalRayProducer *rp) {
  if (!rp || !rp->m_ctx || !rp->m_vol || rp->m_proj < 0) return;
  wap_ctx *c = rp->m_ctx;
  const size_t np = (size_t)rp->m_W * rp->m_H;
  DeviceBuffer img(c, np), len(c, np), wt(c, np);
  check(wap_forward_project(c, rp->m_proj, rp->m_vol->get(), img.get(), len.get(), wt.get()), c,
        "GenerateImage_GetCorrections");
  img.download(rp->m_ImageData, np);
  len.download(rp->m_imageraylength, np);
  wt.download(rp->m_WeightOfImage, np);
}

}  // namespace wap19

#ifdef WAP19_GLOBAL_NAMES
using wap19::CoherentVolume;
using wap19::PSART;
using wap19::VolumeData;
using wap19::Frame_item;
using wap19::TypicalRayProducer;
using wap19::RayCaster;
using wap19::SingleScalarVolumePrepare;
using wap19::RayCasterPrepare;
using wap19::GenerateImage_GetCorrections;
namespace advection = wap19::advection;
namespace optical_flow = wap19::optical_flow;
namespace image_cg = wap19::image_cg;
#endif
