// Per-projection cone-beam geometry on the host.
//
// The reference builds, for every projection, a rotation about +y
// (PSART::RotateVolume, WaP_Tomo.cpp:1764-1797), the view matrix
// T(tx, ty, -sid+tz) * S * R and a GL-style frustum whose near plane is the
// detector (Scene::_calculateCamera / _calculateMatrix, Scene.cpp:65-189),
// then the pixel<->model<->voxel matrices (TypicalRayProducer::_calculateMatrix,
// TypicalRayProducer.cpp:157-232) with a float cofactor inverse
// (Matrix4x4.cpp:80-135).  The forward projector's sample positions depend on
// every bit of these matrices, so the same float operations are performed
// here in the same order; the results are uploaded once per scan.
#include <cmath>
#include <cstring>

#include "wap_geometry.h"

namespace wap {
namespace {

struct Mat {
  float e[16];
  static Mat identity() {
    Mat m;
    for (int i = 0; i < 16; ++i) m.e[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    return m;
  }
};

Mat mul(const Mat &A, const Mat &B) {
  Mat R;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r)
      R.e[4 * c + r] = A.e[r] * B.e[4 * c] + A.e[4 + r] * B.e[4 * c + 1] + A.e[8 + r] * B.e[4 * c + 2] +
                       A.e[12 + r] * B.e[4 * c + 3];
  return R;
}

// 3x3 determinant term order of the reference's Det3x3 macro.
inline float d3(float a, float b, float c, float d, float e, float f, float g, float h, float i) {
  return a * e * i + b * f * g + c * d * h - c * e * g - a * f * h - b * d * i;
}

void invert(Mat &m) {
  float *e = m.e;
  const float a1 = e[0], b1 = e[1], c1 = e[2], dd1 = e[3];
  const float a2 = e[4], b2 = e[5], c2 = e[6], dd2 = e[7];
  const float a3 = e[8], b3 = e[9], c3 = e[10], dd3 = e[11];
  const float a4 = e[12], b4 = e[13], c4 = e[14], dd4 = e[15];
  const float m1 = d3(b2, b3, b4, c2, c3, c4, dd2, dd3, dd4);
  const float m2 = d3(a2, a3, a4, c2, c3, c4, dd2, dd3, dd4);
  const float m3 = d3(a2, a3, a4, b2, b3, b4, dd2, dd3, dd4);
  const float m4 = d3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
  const float det = a1 * m1 - b1 * m2 + c1 * m3 - dd1 * m4;
  if (det == 0.0f) return;
  const float inv = 1.0f / det;
  e[0] = m1 * inv;
  e[4] = -m2 * inv;
  e[8] = m3 * inv;
  e[12] = -m4 * inv;
  e[1] = -d3(b1, b3, b4, c1, c3, c4, dd1, dd3, dd4) * inv;
  e[5] = d3(a1, a3, a4, c1, c3, c4, dd1, dd3, dd4) * inv;
  e[9] = -d3(a1, a3, a4, b1, b3, b4, dd1, dd3, dd4) * inv;
  e[13] = d3(a1, a3, a4, b1, b3, b4, c1, c3, c4) * inv;
  e[2] = d3(b1, b2, b4, c1, c2, c4, dd1, dd2, dd4) * inv;
  e[6] = -d3(a1, a2, a4, c1, c2, c4, dd1, dd2, dd4) * inv;
  e[10] = d3(a1, a2, a4, b1, b2, b4, dd1, dd2, dd4) * inv;
  e[14] = -d3(a1, a2, a4, b1, b2, b4, c1, c2, c4) * inv;
  e[3] = -d3(b1, b2, b3, c1, c2, c3, dd1, dd2, dd3) * inv;
  e[7] = d3(a1, a2, a3, c1, c2, c3, dd1, dd2, dd3) * inv;
  e[11] = -d3(a1, a2, a3, b1, b2, b3, dd1, dd2, dd3) * inv;
  e[15] = d3(a1, a2, a3, b1, b2, b3, c1, c2, c3) * inv;
}

}  // namespace

double half_frustum(int pixels, double ds) { return (pixels - 1) * ds * 0.5f; }

float sample_distance(double vs) {
  const float s = (float)vs;
  return std::sqrt(s * s + s * s + s * s) / 2;
}

ProjGeom projection_geometry(const ScanGeometry &sg, double angle_deg) {
  // Rotation quaternion about +y (WaP_Tomo.cpp:1775-1791; Quaternion.cpp:7-40).
  const double angle = angle_deg * 3.1415926 / 180;
  float axis[3] = {0.0f, 1.0f, 0.0f};
  const double length = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  const float rescale = (float)(1.0f / length);
  for (float &a : axis) a *= rescale;
  const float qangle = (float)(length * angle);
  float qx = 0.0f, qy = 0.0f, qz = 0.0f, qw = 1.0f;
  const float alen = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  if (alen != 0.0f) {
    const float li = 1.0f / alen;
    const float half = qangle / 2;
    const float s = std::sin(half);
    qw = std::cos(half);
    qx = axis[0] * li * s;
    qy = axis[1] * li * s;
    qz = axis[2] * li * s;
  }
  // Composition with the identity reference rotation (Quaternion.h:269-279).
  const float rw = qw * 1.0f - qx * 0.0f - qy * 0.0f - qz * 0.0f;
  const float rx = qw * 0.0f + qx * 1.0f + qy * 0.0f - qz * 0.0f;
  const float ry = qw * 0.0f + qy * 1.0f + qz * 0.0f - qx * 0.0f;
  const float rz = qw * 0.0f + qz * 1.0f + qx * 0.0f - qy * 0.0f;
  Mat R = Mat::identity();
  R.e[0] = 1.0f - 2.0f * (ry * ry + rz * rz);
  R.e[1] = 2.0f * (rx * ry + rz * rw);
  R.e[2] = 2.0f * (rz * rx - ry * rw);
  R.e[4] = 2.0f * (rx * ry - rz * rw);
  R.e[5] = 1.0f - 2.0f * (rz * rz + rx * rx);
  R.e[6] = 2.0f * (ry * rz + rx * rw);
  R.e[8] = 2.0f * (rz * rx + ry * rw);
  R.e[9] = 2.0f * (ry * rz - rx * rw);
  R.e[10] = 1.0f - 2.0f * (rx * rx + ry * ry);
  // View and frustum (Scene.cpp:65-189); Scene keeps sid, sdd as floats.
  const float sid = (float)sg.sid, sdd = (float)sg.sdd;
  const float near_p = sdd, far_p = (float)10000.0;
  Mat T = Mat::identity();
  T.e[12] = (float)(-sg.oxyz[0]);
  T.e[13] = (float)(-sg.oxyz[2]);
  T.e[14] = -1 * sid + (float)(+sg.oxyz[1]);
  const Mat view = mul(mul(T, Mat::identity()), R);
  const double hw = half_frustum(sg.det[0], sg.ds), hh = half_frustum(sg.det[1], sg.ds);
  Mat P;
  std::memset(P.e, 0, sizeof(P.e));
  P.e[0] = (float)(near_p / hw);
  P.e[5] = (float)(near_p / hh);
  P.e[10] = -(far_p + near_p) / (far_p - near_p);
  P.e[11] = -1.0f;
  P.e[14] = -2.0f * far_p * near_p / (far_p - near_p);
  // Model-view with the volume centred (TypicalRayProducer.cpp:118-165).
  const float sp = (float)sg.vs;
  Mat C = Mat::identity();
  for (int a = 0; a < 3; ++a) C.e[12 + a] = -((sg.vol[a] - 1) * sp) * 0.5f;
  const Mat MV = mul(view, C);
  Mat M2V = Mat::identity();
  M2V.e[0] = 1.0f / sp;
  M2V.e[5] = 1.0f / sp;
  M2V.e[10] = 1.0f / sp;
  Mat V2M = M2V;
  invert(V2M);
  Mat V2P;
  std::memset(V2P.e, 0, sizeof(V2P.e));
  V2P.e[0] = 0.5f * (sg.det[0] - 1);
  V2P.e[5] = 0.5f * (sg.det[1] - 1);
  V2P.e[10] = 0.5f;
  V2P.e[12] = V2P.e[0];
  V2P.e[13] = V2P.e[5];
  V2P.e[14] = V2P.e[10];
  V2P.e[15] = 1.0f;
  Mat P2M = mul(mul(V2P, P), MV);
  invert(P2M);
  ProjGeom g;
  std::memcpy(g.p2m, P2M.e, sizeof(g.p2m));
  std::memcpy(g.m2v, M2V.e, sizeof(g.m2v));
  const Mat mvv2m = mul(MV, V2M);
  std::memcpy(g.mvv2m, mvv2m.e, sizeof(g.mvv2m));
  // EyePos (TypicalRayProducer.core.h:255-258).
  g.eye[0] = P2M.e[8] / P2M.e[11];
  g.eye[1] = P2M.e[9] / P2M.e[11];
  g.eye[2] = P2M.e[10] / P2M.e[11];
  g.eye[3] = 1.0f;
  return g;
}

int level_frames(int nframes_cli, int nproj, int level, int *start, int *end, float *ftime, float *tunit, int cap) {
  // VolumeData::ReadStructuredFile (VolumeData.cpp:133-210).
  const int factor = 1 << level;
  const int nf = (nframes_cli * factor < 130) ? nframes_cli * factor : 130;
  const float unit = (float)((float)nproj / (float)nf);
  const float base = 3;
  for (int i = 0; i < nf && i < cap; ++i) {
    const float t = unit * i;
    if (ftime) ftime[i] = t;
    const int s = (int)(t - base), e = (int)(t + base);
    if (start) start[i] = s > 0 ? s : 0;
    if (end) end[i] = e < nproj - 1 ? e : nproj - 1;
  }
  if (tunit) *tunit = unit;
  return nf;
}

}  // namespace wap
