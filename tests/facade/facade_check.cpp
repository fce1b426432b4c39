// Exercises the C++ facade (include/wap/wap19.hpp) with the reference's
// names, on files written by tests/test_facade_gpu.py:
//   facade_check advect  <vel.hdr> <src.hdr> <dt> <out.hdr>
//   facade_check flow    <I1.hdr> <I2.hdr> <V0.hdr> <iters> <scales> <cut> <out.hdr>
//   facade_check level   <I1.hdr> <I2.hdr> <V0.hdr> <iters> <roi> <outV.hdr>
//   facade_check cg      <rhs.hdr> <a> <b> <iters> <out.hdr>
//   facade_check project <vol.hdr> <W> <H> <nproj> <proj> <sid> <sdd> <angles.txt> <out.hdr>
// The image type is a template parameter, as in the reference's headers; the
// build also instantiates everything with CImg<float> when the reference's
// CImg.h is on the include path (-DWAP_WITH_CIMG).
#include <cstdlib>
#include <cstdio>
#include <string>

#define WAP19_GLOBAL_NAMES
#include "wap/wap19.hpp"

#ifdef WAP_WITH_CIMG
#define cimg_display 0
#include "CImg.h"
template void wap19::image_cg::cg<float, cimg_library::CImg<float>, wap19::image_cg::ScreenedLaplacian>(
    wap19::image_cg::ScreenedLaplacian &, cimg_library::CImg<float> &, const cimg_library::CImg<float> &, float, int,
    float);
template cimg_library::CImg<float> wap19::advection::advect<float, cimg_library::CImg<float>>(
    const int *, const float *, const cimg_library::CImg<float> &, const cimg_library::CImg<float> &, float);
template cimg_library::CImg<float> wap19::optical_flow::L1TVOpticalFlowNonlinear_MultiScale3D<
    float, cimg_library::CImg<float>>(int *, const cimg_library::CImg<float> &, const cimg_library::CImg<float> &,
                                      cimg_library::CImg<float> &, cimg_library::CImg<float> &,
                                      cimg_library::CImg<float> &, cimg_library::CImg<float> &,
                                      cimg_library::CImg<float> &, float, float, int, int, int, float, float, int,
                                      float, int *);
#endif

using wap19::Image;

int main(int argc, char **argv) {
  if (argc < 2) return 1;
  const std::string cmd = argv[1];
  try {
    if (cmd == "advect" && argc == 6) {
      Image vel = Image::load_analyze(argv[2]), src = Image::load_analyze(argv[3]);
      int dim[3] = {src.width(), src.height(), src.depth()};
      float aabb[6] = {0, (float)dim[0], 0, (float)dim[1], 0, (float)dim[2]};
      Image out = advection::advect<float, Image>(dim, aabb, vel, src, (float)std::atof(argv[4]));
      out.save_analyze(argv[5]);
    } else if (cmd == "flow" && argc == 9) {
      Image I1 = Image::load_analyze(argv[2]), I2 = Image::load_analyze(argv[3]), V = Image::load_analyze(argv[4]);
      int dim[3] = {I1.width(), I1.height(), I1.depth()};
      Image Y1(dim[0], dim[1], dim[2], 3), Y2(dim[0], dim[1], dim[2], 3), Y3(dim[0], dim[1], dim[2], 3),
          Y4(dim[0], dim[1], dim[2], 1);
      const int c = std::atoi(argv[7]);
      int cut[8] = {c, c, c, c, c, c, c, c};
      Image out = optical_flow::L1TVOpticalFlowNonlinear_MultiScale3D<float, Image>(
          dim, I1, I2, V, Y1, Y2, Y3, Y4, 0.0f, 0.05f, std::atoi(argv[5]), 1, 2, 0.5f, 0.8f, std::atoi(argv[6]), 1.0f,
          cut);
      out.save_analyze(argv[8]);
    } else if (cmd == "level" && argc == 8) {
      Image I1 = Image::load_analyze(argv[2]), I2 = Image::load_analyze(argv[3]), V = Image::load_analyze(argv[4]);
      int dim[3] = {I1.width(), I1.height(), I1.depth()};
      Image Y1(dim[0], dim[1], dim[2], 3), Y2(dim[0], dim[1], dim[2], 3), Y3(dim[0], dim[1], dim[2], 3),
          Y4(dim[0], dim[1], dim[2], 1);
      const int r = std::atoi(argv[6]);
      int roi[6] = {r, r, r, r, r, r};
      float aabb[6] = {0, (float)dim[0], 0, (float)dim[1], 0, (float)dim[2]};
      optical_flow::L1TVOpticalFlowNonlinear3D<float, Image>(dim, I1, I2, V, Y1, Y2, Y3, Y4, 0.0f, 0.05f,
                                                             std::atoi(argv[5]), 1, 2, aabb, 1.0f, roi);
      V.save_analyze(argv[7]);
    } else if (cmd == "cg" && argc == 7) {
      Image b = Image::load_analyze(argv[2]);
      Image x(b.width(), b.height(), b.depth(), 1, 0.0f);
      image_cg::ScreenedLaplacian A;
      A.a = (float)std::atof(argv[3]);
      A.b = (float)std::atof(argv[4]);
      A.mode = 1;
      image_cg::cg<float, Image, image_cg::ScreenedLaplacian>(A, x, b, 1e-5f, std::atoi(argv[5]), 1e-9f);
      x.save_analyze(argv[6]);
    } else if (cmd == "project" && argc == 11) {
      Image vol = Image::load_analyze(argv[2]);
      int vols[3] = {vol.width(), vol.height(), vol.depth()};
      int wh[2] = {std::atoi(argv[3]), std::atoi(argv[4])};
      const int np = std::atoi(argv[5]), proj = std::atoi(argv[6]);
      double oxyz[3] = {0, 0, 0}, sdg[1] = {0};
      const char *pf[1] = {nullptr};
      VolumeData data;
      data.setParas(vols, 1.0, 1, np);
      data.ReadStructuredFile(1);
      PSART scene(0.3, 0.3, 0.1, "unused", wh, np, 2, 2, 0.1, std::atof(argv[7]), pf, oxyz, std::atof(argv[8]), 1.0,
                  "ATV", "Voxelbased", vols, 1, sdg, 1, argv[9]);
      scene.SetData(&data);
      data.m_Frameslist[0][0].fVolume = vol;
      RayCaster rc;
      SingleScalarVolumePrepare(&data, scene.m_RayProducer, 0, false, proj, 0.0f, 0);
      RayCasterPrepare(&rc, vols);
      GenerateImage_GetCorrections(scene.m_RayProducer);
      Image out(wh[0], wh[1], 1, 3);
      const size_t n = (size_t)wh[0] * wh[1];
      std::memcpy(out.data(), scene.m_RayProducer->m_ImageData, n * 4);
      std::memcpy(out.data() + n, scene.m_RayProducer->m_imageraylength, n * 4);
      std::memcpy(out.data() + 2 * n, scene.m_RayProducer->m_WeightOfImage, n * 4);
      out.save_analyze(argv[10]);
    } else {
      std::fprintf(stderr, "bad arguments\n");
      return 1;
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "facade_check: %s\n", e.what());
    return 2;
  }
  return 0;
}
