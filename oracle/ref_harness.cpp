// Oracle build only (test infrastructure, never shipped or timed).
//
// Drives the reference's OWN sources -- compiled from where they lie in the
// reference tree by oracle/Makefile -- through a few C entry points, so the
// parity tests can pin the oracle restatement (oracle/wap_oracle.cpp) against
// the reference itself.  Nothing here restates an algorithm: every number this
// library returns is computed by reference code (PSART, GenerateImage_GetCorrections,
// advection::advect, optical_flow::*, image_cg::cg, CImg).
//
// Parity-defining choices applied to the reference (the reference is undefined
// or crashes without them):
//   * every frame's flow starts as a zero 3-channel field (an empty CImg makes
//     advect and the flow solver dereference null data: WaP_Tomo.cpp:749,
//     SingleScalarVolume.core.h:399-402);
//   * VolumeData::m_roi is zero when PSART::SetData runs (WaP_Tomo.cpp:391-417
//     reads it uninitialised) -> imROI == 1;
//   * `new T[]` returns zeroed memory inside this library, so the flow
//     solver's never-written ux/uy/uz/ut outside the ROI read as 0
//     (optical_flow.h:181-184,426-445);
//   * the PSART dual pY gets one row per projection id (shim Eigen/Core);
//   * exit(0) at the end of PSART::Render is turned into an exception.
#include <cmath>
#include <cstdio>
#include <ctime>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>
#include <new>
#include <omp.h>
#include <sys/stat.h>
#include <unistd.h>

#define private public
#define protected public
#include "WaP_Tomo.cpp"
#include "CoherentVolume.h"
#undef private
#undef protected

extern bool isRaybased;  // TypicalRayProducer.cpp:24

void *operator new[](std::size_t n) {
  void *p = std::calloc(n ? n : 1, 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void operator delete[](void *p) noexcept { std::free(p); }
void operator delete[](void *p, std::size_t) noexcept { std::free(p); }

namespace {

struct Session {
  VolumeData *data = nullptr;
  PSART *scene = nullptr;
  std::string dir;
  int W = 0, H = 0, P = 0;
  int dims[3] = {0, 0, 0};
  std::vector<const char *> files;
  std::string projfile;
  std::string outprefix;
};

Session g;
std::streambuf *g_cout_saved = nullptr;

struct QuietCout {
  QuietCout() { g_cout_saved = std::cout.rdbuf(nullptr); }
  ~QuietCout() { std::cout.rdbuf(g_cout_saved); std::cout.clear(); }
};

struct InDir {
  char old[4096];
  InDir(const std::string &d) {
    if (!getcwd(old, sizeof(old))) old[0] = 0;
    if (chdir(d.c_str()) != 0) throw std::runtime_error("chdir failed");
  }
  ~InDir() {
    if (old[0] && chdir(old) != 0) {}
  }
};

void mk(const std::string &p) { mkdir(p.c_str(), 0755); }

image &frame_vol(int level, int frame) { return g.data->m_Frameslist[level][frame].fVolume; }
image &frame_flow(int level, int frame) { return g.data->m_Frameslist[level][frame].fFlow; }

void set_roi_from_cut() {
  // PSART::Render:529-536 with cut = 8 and level-0 size == volume size.
  for (int i = 0; i < 8; ++i) {
    int axis = (i < 2) ? 0 : (i < 4) ? 1 : 2;
    if (i >= 6) axis = 2;
    g.data->m_roi[i] = (float)cut[i] * ((float)g.dims[axis] / (float)g.data->m_Volumesize[0].volsize[axis]);
  }
}

void ensure_dual_rows() {
  pY_warp = Eigen::MatrixXf::Zero(1, PRO_WIDTH * PRO_HEIGHT);
  pY_Adaptive = Eigen::MatrixXf::Zero(1, PRO_WIDTH * PRO_HEIGHT);
  pY = Eigen::MatrixXf::Zero(PRO_NO, PRO_WIDTH * PRO_HEIGHT);
}

}  // namespace

extern "C" {

// Builds VolumeData + PSART exactly as main.cpp:195-219 does (GLUT window and
// file I/O replaced by in-memory data).  projs: W*H*P floats, CImg layout
// (x fastest, one projection per z slice); angles_deg: P doubles.
int wref_create(int vx, int vy, int vz, int W, int H, int P, int nframes_cli, double vs, double ds,
                double sid, double sdd, double alpha, double tv_w, double tp_w, const double *oxyz,
                const float *projs, const double *angles_deg, const char *workdir) {
  QuietCout q;
  try {
    g = Session();
    g.dir = workdir;
    mk(g.dir);
    mk(g.dir + "/WarpStep");
    mk(g.dir + "/warpedVolume");
    mk(g.dir + "/VelocityField");
    mk(g.dir + "/out");
    g.W = W;
    g.H = H;
    g.P = P;
    g.dims[0] = vx;
    g.dims[1] = vy;
    g.dims[2] = vz;
    image stack(W, H, P, 1);
    std::memcpy(stack.data(), projs, sizeof(float) * (size_t)W * H * P);
    g.projfile = g.dir + "/projs.cimg";
    stack.save_cimg(g.projfile.c_str());
    g.files.assign(1000, g.projfile.c_str());
    g.outprefix = g.dir + "/out/test";

    int vols[3] = {vx, vy, vz};
    int imgwh[2] = {W, H};
    double off[3] = {oxyz ? oxyz[0] : 0.0, oxyz ? oxyz[1] : 0.0, oxyz ? oxyz[2] : 0.0};
    double startdg[20] = {0};
    g.data = new VolumeData;
    g.data->setParas(vols, vs, nframes_cli, P);
    g.data->ReadStructuredFile();
    for (int l = 0; l < 5; ++l)
      for (auto &f : g.data->m_Frameslist[l]) f.fFlow = image(vx, vy, vz, 3, 0.0f);
    for (int i = 0; i < 8; ++i) g.data->m_roi[i] = 0;
    projslevel[0].assign();
    isRaybased = false;
    {
      InDir d(g.dir);
      g.scene = new PSART(tv_w, tp_w, 0.1, g.outprefix.c_str(), imgwh, P, 2, 2, alpha, sid, g.files.data(), off,
                          sdd, ds, "ATV", "Voxelbased", vols, nframes_cli, startdg, 1);
    }
    for (int i = 0; i < P; ++i) inputdegree[i] = angles_deg[i];
    g.scene->SetData(g.data);
    g.scene->Resize(W, H);
    ensure_dual_rows();
    return 0;
  } catch (...) {
    return -1;
  }
}

void wref_destroy() {
  delete g.scene;
  delete g.data;
  g = Session();
}

float wref_gmax() { return G_Max; }

int wref_level_info(int level, int *nframes, float *tunit) {
  *nframes = g.data->m_fInLevel[level];
  *tunit = g.data->m_tUnitInLevel[level];
  return (int)g.data->m_Frameslist[level].size();
}

int wref_frame_info(int level, int frame, int *start, int *end, float *time) {
  const Frame_item &f = g.data->m_Frameslist[level][frame];
  *start = f.fStartproj;
  *end = f.fEndproj;
  *time = f.fTime;
  return 0;
}

int wref_set_volume(int level, int frame, const float *v) {
  image &im = frame_vol(level, frame);
  std::memcpy(im.data(), v, sizeof(float) * im.size());
  return 0;
}

int wref_get_volume(int level, int frame, float *v) {
  const image &im = frame_vol(level, frame);
  std::memcpy(v, im.data(), sizeof(float) * im.size());
  return 0;
}

int wref_set_flow(int level, int frame, const float *v) {
  image &im = frame_flow(level, frame);
  std::memcpy(im.data(), v, sizeof(float) * im.size());
  return 0;
}

int wref_get_flow(int level, int frame, float *v) {
  const image &im = frame_flow(level, frame);
  if (im.is_empty()) return -1;
  std::memcpy(v, im.data(), sizeof(float) * im.size());
  return 0;
}

// The per-projection matrices PSART::RotateVolume + Scene::_calculateCamera/
// _calculateMatrix + TypicalRayProducer::_calculateMatrix produce
// (WaP_Tomo.cpp:1764-1797, Scene.cpp:65-189, TypicalRayProducer.cpp:157-232).
int wref_geometry(int proj, float *p2m, float *m2v, float *mv, float *v2m, float *eye) {
  QuietCout q;
  PSART *s = g.scene;
  s->RotateVolume(proj);
  s->_calculateCamera();
  s->_calculateMatrix();
  s->m_RayProducer->SetViewMatrix(s->GetViewMatrix());
  s->m_RayProducer->SetProjectionMatrix(s->GetProjectionMatrix());
  s->m_RayProducer->UpdateMatrixAndBounds();
  std::memcpy(p2m, s->m_RayProducer->m_PixelsToModelMatrix.ele, 64);
  std::memcpy(m2v, s->m_RayProducer->m_ModelToVolumeMatrix.ele, 64);
  std::memcpy(mv, s->m_RayProducer->m_model_view.ele, 64);
  std::memcpy(v2m, s->m_RayProducer->m_VolumeToModelMatrix.ele, 64);
  const Matrix4x4 &P2M = s->m_RayProducer->m_PixelsToModelMatrix;
  eye[0] = P2M[8] / P2M[11];
  eye[1] = P2M[9] / P2M[11];
  eye[2] = P2M[10] / P2M[11];
  eye[3] = 1.0f;
  return 0;
}

// One forward projection of frame `frame` at projection `proj`, warped by the
// frame's flow when warped != 0 (PSART::RenderContent -> _renderCoreFuc ->
// GenerateImage_GetCorrections).  Outputs W*H floats each.
int wref_forward(int level, int frame, int proj, int warped, float rtime, float *img, float *len, float *weight) {
  QuietCout q;
  PSART *s = g.scene;
  s->RotateVolume(proj);
  s->_calculateCamera();
  s->_calculateMatrix();
  s->m_NeedCalculateCamera = false;
  s->m_NeedCalculateMatrix = false;
  s->RenderContent(frame, warped != 0, proj, rtime, level);
  size_t n = (size_t)g.W * g.H;
  std::memcpy(img, s->m_RayProducer->m_ImageData, n * 4);
  std::memcpy(len, s->m_RayProducer->m_imageraylength, n * 4);
  std::memcpy(weight, s->m_RayProducer->m_WeightOfImage, n * 4);
  s->m_RayProducer->Initial();
  return 0;
}

// The dead ray-driven backprojection path (SingleScalarVolume.core.h:85-96,
// 149-199), reached by switching VolumeData into back-projection mode.  Runs
// single-threaded: the reference's += on shared voxels races under OpenMP.
int wref_ray_backproject(int level, int frame, int proj, const float *correction, float *contrib, float *weight) {
  QuietCout q;
  PSART *s = g.scene;
  size_t n = (size_t)g.W * g.H;
  size_t nv = (size_t)g.dims[0] * g.dims[1] * g.dims[2];
  int saved = omp_get_max_threads();
  omp_set_num_threads(1);
  std::memset(s->m_RayProducer->m_Voxel_Contributions, 0, nv * 4);
  std::memset(s->m_RayProducer->m_EachVoxel_TotalWeight, 0, nv * 4);
  std::memcpy(s->m_RayProducer->m_Correction, correction, n * 4);
  g.data->SetProjectionMode(true);
  s->RotateVolume(proj);
  s->_calculateCamera();
  s->_calculateMatrix();
  s->RenderContent(frame, false, proj, 0.0f, level);
  g.data->SetProjectionMode(false);
  std::memcpy(contrib, s->m_RayProducer->m_Voxel_Contributions, nv * 4);
  std::memcpy(weight, s->m_RayProducer->m_EachVoxel_TotalWeight, nv * 4);
  s->m_RayProducer->Initial();
  omp_set_num_threads(saved);
  return 0;
}

// PSART::SART_Proximal_Operator (WaP_Tomo.cpp:1424-1678) on one frame; the
// ROI box comes from the cut the way Render sets it (WaP_Tomo.cpp:529-536)
// unless use_cut == 0 (then the whole volume).
int wref_sart_prox(int level, int frame, int nb_sart, int use_cut) {
  QuietCout q;
  try {
    if (use_cut) set_roi_from_cut();
    else for (int i = 0; i < 8; ++i) g.data->m_roi[i] = 0;
    InDir d(g.dir);
    g.scene->SART_Proximal_Operator(frame, nb_sart, 0, 1, level);
    return 0;
  } catch (...) {
    return -1;
  }
}

// PSART::WarpAndProjct (WaP_Tomo.cpp:1207-1421) for one projection.
int wref_warp_and_project(int level, int frame, int proj, float rtime) {
  QuietCout q;
  try {
    int dims[3] = {g.dims[0], g.dims[1], g.dims[2]};
    float aabb[6] = {0, (float)dims[0], 0, (float)dims[1], 0, (float)dims[2]};
    char head[] = "WarpStep";
    InDir d(g.dir);
    g.scene->WarpAndProjct(proj, frame, dims, rtime, aabb, 0, 0, head, level);
    return 0;
  } catch (...) {
    return -1;
  }
}

// One complete PSART::Render (WaP_Tomo.cpp:473-877) with the reference's
// hard-coded schedule.  Returns 0 when Render reached its exit(0).
int wref_render() {
  QuietCout q;
  try {
    InDir d(g.dir);
    g.scene->Render();
    return -2;
  } catch (const wap_ref_exit_signal &) {
    return 0;
  } catch (...) {
    return -1;
  }
}

// advection::advect<float> (advection.h:118-146).  vel: 3 planar channels,
// src/out: nc planar channels, all dims[0]*dims[1]*dims[2] per channel.
int wref_advect(const int *dims, const float *aabb, const float *vel, const float *src, int nc, float dt, float *out) {
  image V(dims[0], dims[1], dims[2], 3), S(dims[0], dims[1], dims[2], nc);
  std::memcpy(V.data(), vel, V.size() * 4);
  std::memcpy(S.data(), src, S.size() * 4);
  int d[3] = {dims[0], dims[1], dims[2]};
  image o = advection::advect<float, image>(d, aabb, V, S, dt);
  std::memcpy(out, o.data(), o.size() * 4);
  return 0;
}

// CImg::get_blur(sigma) (Deriche order 0, Neumann; CImg.h:33249-33285).
int wref_blur(const int *dims, int nc, float sigma, const float *src, float *out) {
  image S(dims[0], dims[1], dims[2], nc);
  std::memcpy(S.data(), src, S.size() * 4);
  image o = S.get_blur(sigma);
  std::memcpy(out, o.data(), o.size() * 4);
  return 0;
}

// CImg::get_resize(..., interpolation 5) as the flow pyramid calls it
// (optical_flow.h:1036-1052,1101-1115).
int wref_resize(const int *dims, int nc, const float *src, const int *odims, float *out) {
  image S(dims[0], dims[1], dims[2], nc);
  std::memcpy(S.data(), src, S.size() * 4);
  image o = S.get_resize(odims[0], odims[1], odims[2], nc, interpo);
  std::memcpy(out, o.data(), o.size() * 4);
  return 0;
}

// CImg::get_gradient("xyz", 0): centred differences (CImg.h:34570-34590).
int wref_gradient(const int *dims, const float *src, float *gx, float *gy, float *gz) {
  image S(dims[0], dims[1], dims[2], 1);
  std::memcpy(S.data(), src, S.size() * 4);
  imagelist gl = S.get_gradient("xyz", 0);
  std::memcpy(gx, gl[0].data(), S.size() * 4);
  std::memcpy(gy, gl[1].data(), S.size() * 4);
  std::memcpy(gz, gl[2].data(), S.size() * 4);
  return 0;
}

// optical_flow::L1TVOpticalFlowNonlinear3D (optical_flow.h:88-995): one
// pyramid level, V (3 ch) and Y1..Y3 (3 ch), Y4 (1 ch) updated in place.
int wref_flow_level(const int *dims, const float *I1, const float *I2, float *V, float *Y1, float *Y2, float *Y3,
                    float *Y4, float tol, float lambda, int max_iters, int nwarps, const float *aabb,
                    const int *roi6) {
  QuietCout q;
  int d[3] = {dims[0], dims[1], dims[2]};
  image i1(d[0], d[1], d[2], 1), i2(d[0], d[1], d[2], 1), v(d[0], d[1], d[2], 3), y1(d[0], d[1], d[2], 3),
      y2(d[0], d[1], d[2], 3), y3(d[0], d[1], d[2], 3), y4(d[0], d[1], d[2], 1);
  std::memcpy(i1.data(), I1, i1.size() * 4);
  std::memcpy(i2.data(), I2, i2.size() * 4);
  std::memcpy(v.data(), V, v.size() * 4);
  std::memcpy(y1.data(), Y1, y1.size() * 4);
  std::memcpy(y2.data(), Y2, y2.size() * 4);
  std::memcpy(y3.data(), Y3, y3.size() * 4);
  std::memcpy(y4.data(), Y4, y4.size() * 4);
  float ab[6];
  std::memcpy(ab, aabb, sizeof(ab));
  int roi[6];
  std::memcpy(roi, roi6, sizeof(roi));
  optical_flow::L1TVOpticalFlowNonlinear3D<float, image>(d, i1, i2, v, y1, y2, y3, y4, tol, lambda, max_iters, 1,
                                                          nwarps, ab, 1.0f, roi);
  std::memcpy(V, v.data(), v.size() * 4);
  std::memcpy(Y1, y1.data(), y1.size() * 4);
  std::memcpy(Y2, y2.data(), y2.size() * 4);
  std::memcpy(Y3, y3.data(), y3.size() * 4);
  std::memcpy(Y4, y4.data(), y4.size() * 4);
  return 0;
}

// optical_flow::L1TVOpticalFlowNonlinear_MultiScale3D (optical_flow.h:1002-1126)
// as PSART::Render calls it (WaP_Tomo.cpp:711-753): Y1..Y4 start at zero,
// V0 is the warm start; the finest-level flow is written to Vout.
int wref_flow_multiscale(const int *dims, const float *I1, const float *I2, const float *V0, float tol, float lambda,
                         int max_iters, int nwarps, float eta, float sigma, int scales, const int *cut6,
                         float *Vout) {
  QuietCout q;
  int d[3] = {dims[0], dims[1], dims[2]};
  image i1(d[0], d[1], d[2], 1), i2(d[0], d[1], d[2], 1), v(d[0], d[1], d[2], 3);
  std::memcpy(i1.data(), I1, i1.size() * 4);
  std::memcpy(i2.data(), I2, i2.size() * 4);
  std::memcpy(v.data(), V0, v.size() * 4);
  image y1(d[0], d[1], d[2], 3, 0.0f), y2(d[0], d[1], d[2], 3, 0.0f), y3(d[0], d[1], d[2], 3, 0.0f),
      y4(d[0], d[1], d[2], 1, 0.0f);
  int c[8];
  for (int i = 0; i < 6; ++i) c[i] = cut6[i];
  c[6] = c[7] = 0;
  image o = optical_flow::L1TVOpticalFlowNonlinear_MultiScale3D<float, image>(
      d, i1, i2, v, y1, y2, y3, y4, tol, lambda, max_iters, 1, nwarps, eta, sigma, scales, 1.0f, c);
  std::memcpy(Vout, o.data(), o.size() * 4);
  return 0;
}

}  // extern "C"

namespace {
// A screened-Poisson operator A x = a*x - b*Lap(x) with Neumann (clamped)
// neighbours, used to exercise image_cg::cg (cg.h has no caller in the
// reference, so the operator is the test's choice).
struct ScreenedLaplacian {
  float a, b;
  void operator()(const image &x, image &y) const {
    y.assign(x.width(), x.height(), x.depth(), x.spectrum());
    const int W = x.width(), H = x.height(), D = x.depth();
    for (int c = 0; c < x.spectrum(); ++c)
      for (int k = 0; k < D; ++k)
        for (int j = 0; j < H; ++j)
          for (int i = 0; i < W; ++i) {
            float xc = x(i, j, k, c);
            float s = x(i > 0 ? i - 1 : i, j, k, c) + x(i < W - 1 ? i + 1 : i, j, k, c) +
                      x(i, j > 0 ? j - 1 : j, k, c) + x(i, j < H - 1 ? j + 1 : j, k, c) +
                      x(i, j, k > 0 ? k - 1 : k, c) + x(i, j, k < D - 1 ? k + 1 : k, c);
            y(i, j, k, c) = a * xc - b * (s - 6.0f * xc);
          }
  }
};
}  // namespace

extern "C" {
// image_cg::cg<float> (cg.h:11-55) on the screened Laplacian above.
int wref_cg_screened_laplacian(const int *dims, float a, float b, const float *rhs, float *x, float rel_tol,
                               int max_iters, float abs_tol) {
  QuietCout q;
  image X(dims[0], dims[1], dims[2], 1), B(dims[0], dims[1], dims[2], 1);
  std::memcpy(X.data(), x, X.size() * 4);
  std::memcpy(B.data(), rhs, B.size() * 4);
  ScreenedLaplacian A{a, b};
  image_cg::cg<float, image, ScreenedLaplacian>(A, X, B, rel_tol, max_iters, abs_tol);
  std::memcpy(x, X.data(), X.size() * 4);
  return 0;
}
}

extern "C" {
// CImg<float>::save_analyze (CImg.h:51715-51790), the writer of every
// reference output volume.
int wref_save_analyze(const char *path, const float *data, const int *dims4) {
  image I(dims4[0], dims4[1], dims4[2], dims4[3]);
  std::memcpy(I.data(), data, I.size() * 4);
  try {
    I.save_analyze(path);
  } catch (...) {
    return -1;
  }
  return 0;
}

// CImg<float> load of an Analyze/NIfTI file (CImg.h:47829-47955), the loader
// behind PSART's `image(pInput[0])` (WaP_Tomo.cpp:339).  dims4 gets W,H,D,C.
int wref_load_analyze(const char *path, float *out, long long cap, int *dims4) {
  image I;
  try {
    I.load_analyze(path);
  } catch (...) {
    return -1;
  }
  dims4[0] = I.width();
  dims4[1] = I.height();
  dims4[2] = I.depth();
  dims4[3] = I.spectrum();
  if ((long long)I.size() > cap) return -2;
  std::memcpy(out, I.data(), I.size() * 4);
  return 0;
}

// CImg::get_split('z', nb) on a 1x1xdepth ramp: first slice and slice count
// of each piece (CImg.h:31389-31431).
int wref_split_z(int depth, int nb, int *first, int *count) {
  image I(1, 1, depth, 1);
  for (int k = 0; k < depth; ++k) I(0, 0, k) = (float)k;
  imagelist L;
  try {
    L = I.get_split('z', nb);
  } catch (...) {
    return -1;
  }
  for (int k = 0; k < (int)L.size(); ++k) {
    first[k] = (int)L[k](0, 0, 0);
    count[k] = L[k].depth();
  }
  return (int)L.size();
}
}

extern "C" {
// The reference's CoherentVolume (CoherentVolume.cpp:33-258) on a volume of
// one block per axis (the case its byte-scaled pointer steps leave defined):
// every GetValue, the block range from GetMinMaxValue.
int wref_coherent_volume(const int bs[3], const int dims[3], float *data, float *values, double *minmax) {
  CoherentVolume cv(bs[0], bs[1], bs[2]);
  cv.SetDimensions(dims);
  int bn[3];
  cv.GetBlockNum(bn);
  if (bn[0] != 1 || bn[1] != 1 || bn[2] != 1) return -1;
  cv.AllocateBlocks();
  cv.SetData(data);
  for (int z = 0; z < dims[2]; ++z)
    for (int y = 0; y < dims[1]; ++y)
      for (int x = 0; x < dims[0]; ++x) values[x + dims[0] * (y + dims[1] * z)] = cv.GetValue(x, y, z);
  cv.GetMinMaxValue(minmax[0], minmax[1]);
  return 0;
}
}
