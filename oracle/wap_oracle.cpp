// CPU oracle for the warp-and-project hot path -- TEST INFRASTRUCTURE ONLY.
//
// A restatement of the reference's CPU algorithm in plain C++/OpenMP.  It is
// the checker for the GPU product (tests/, smoke(), bench.py's CPU baseline)
// and is never linked into the product.  Compiled with -ffp-contract=off so
// every real operation rounds where the reference's does.  The
// parity-defining choices for the reference's undefined spots are:
//   * one PSART dual row per projection id, zeroed per SART call;
//   * imROI == 1 (m_roi is zero when SetData builds it);
//   * a frame whose flow was never computed uses a zero field;
//   * flow-solver arrays never written outside the ROI read as 0;
//   * CP state is one channel (only channel 0 of the reference's 3-channel
//     Y_tp / X_bar lists is ever read; Y_bc stays 0).
#include "wap_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// float or double: see orc_real in wap_oracle.h.
typedef orc_real real;

// ---------------------------------------------------------------------------
// 4x4 real matrices, column-major (Matrix4x4.h / Matrix4x4.cpp semantics)
// ---------------------------------------------------------------------------
struct M4 {
  real e[16];
};

M4 m4_identity() {
  M4 m;
  for (int i = 0; i < 16; ++i) m.e[i] = (i % 5 == 0) ? 1.0f : 0.0f;
  return m;
}

// Matrix4x4.h operator*(A,B): each entry summed left to right over k.
M4 m4_mul(const M4 &A, const M4 &B) {
  M4 R;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r)
      R.e[4 * c + r] = A.e[r] * B.e[4 * c] + A.e[4 + r] * B.e[4 * c + 1] + A.e[8 + r] * B.e[4 * c + 2] +
                       A.e[12 + r] * B.e[4 * c + 3];
  return R;
}

// Matrix4x4.h operator*(Mat, Vec).
void m4_vec(const real *M, const real v[4], real out[4]) {
  for (int r = 0; r < 4; ++r) out[r] = M[r] * v[0] + M[4 + r] * v[1] + M[8 + r] * v[2] + M[12 + r] * v[3];
}

inline real det3(real a, real b, real c, real d, real e, real f, real g, real h, real i) {
  return a * e * i + b * f * g + c * d * h - c * e * g - a * f * h - b * d * i;
}

// Cofactor inverse, Matrix4x4.cpp:80-135 (returns unchanged when singular).
void m4_inverse(M4 &m) {
  real *e = m.e;
  real a1 = e[0], b1 = e[1], c1 = e[2], d1 = e[3];
  real a2 = e[4], b2 = e[5], c2 = e[6], d2 = e[7];
  real a3 = e[8], b3 = e[9], c3 = e[10], d3 = e[11];
  real a4 = e[12], b4 = e[13], c4 = e[14], d4 = e[15];
  real det1 = det3(b2, b3, b4, c2, c3, c4, d2, d3, d4);
  real det2 = det3(a2, a3, a4, c2, c3, c4, d2, d3, d4);
  real det3_ = det3(a2, a3, a4, b2, b3, b4, d2, d3, d4);
  real det4 = det3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
  real det = a1 * det1 - b1 * det2 + c1 * det3_ - d1 * det4;
  if (det == 0.0f) return;
  real invdet = 1.0f / det;
  e[0] = det1 * invdet;
  e[4] = -det2 * invdet;
  e[8] = det3_ * invdet;
  e[12] = -det4 * invdet;
  e[1] = -det3(b1, b3, b4, c1, c3, c4, d1, d3, d4) * invdet;
  e[5] = det3(a1, a3, a4, c1, c3, c4, d1, d3, d4) * invdet;
  e[9] = -det3(a1, a3, a4, b1, b3, b4, d1, d3, d4) * invdet;
  e[13] = det3(a1, a3, a4, b1, b3, b4, c1, c3, c4) * invdet;
  e[2] = det3(b1, b2, b4, c1, c2, c4, d1, d2, d4) * invdet;
  e[6] = -det3(a1, a2, a4, c1, c2, c4, d1, d2, d4) * invdet;
  e[10] = det3(a1, a2, a4, b1, b2, b4, d1, d2, d4) * invdet;
  e[14] = -det3(a1, a2, a4, b1, b2, b4, c1, c2, c4) * invdet;
  e[3] = -det3(b1, b2, b3, c1, c2, c3, d1, d2, d3) * invdet;
  e[7] = det3(a1, a2, a3, c1, c2, c3, d1, d2, d3) * invdet;
  e[11] = -det3(a1, a2, a3, b1, b2, b3, d1, d2, d3) * invdet;
  e[15] = det3(a1, a2, a3, b1, b2, b3, c1, c2, c3) * invdet;
}

// The reference's min/max macros (RayCaster.core.h:22-28, WaP_Tomo.cpp:170-176).
template <class A, class B>
inline auto mac_min(A a, B b) {
  return (a < b) ? a : b;
}
template <class A, class B>
inline auto mac_max(A a, B b) {
  return (a > b) ? a : b;
}
// std::min / std::max argument order (used by advection.h, optical_flow.h).
inline real std_min(real a, real b) { return (b < a) ? b : a; }
inline real std_max(real a, real b) { return (a < b) ? b : a; }

struct ProjGeom {
  M4 p2m, m2v, mv, v2m, mvv2m;
  real eye[4];
};

// PSART::RotateVolume + Scene::_calculateCamera/_calculateMatrix +
// TypicalRayProducer::_calculateMatrix + the EyePos of
// GenerateImage_GetCorrections.
ProjGeom make_geometry(const orc_scan *s, double angle_deg) {
  ProjGeom g;
  // WaP_Tomo.cpp:1775-1791: quaternion about +y (IS_COUNTERCLOCK = 1).
  double angle = angle_deg * 3.1415926 / 180;
  real v[4] = {0.0f, 1.0f, 0.0f, 0.0f};
  double length = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);  // sqrtf: all operands real
  real sc = (real)(1.0f / length);
  for (int i = 0; i < 4; ++i) v[i] *= sc;
  real qang = (real)(length * angle);
  // Quaternion.cpp:7-40
  real ax = v[0], ay = v[1], az = v[2];
  real qlen = std::sqrt(ax * ax + ay * ay + az * az);
  real qx, qy, qz, qw;
  if (0.0f == qlen) {
    qw = 1.0f;
    qx = qy = qz = 0.0f;
  } else {
    real lenInv = 1.0f / qlen;
    real xx = ax * lenInv, yy = ay * lenInv, zz = az * lenInv;
    real rad = qang / 2;
    qw = std::cos(rad);
    real scale = std::sin(rad);
    qx = xx * scale;
    qy = yy * scale;
    qz = zz * scale;
  }
  // q * identity (Quaternion.h:269-279 with m_OldRotation = identity).
  real ow = 1.0f, ox = 0.0f, oy = 0.0f, oz = 0.0f;
  real rw = qw * ow - qx * ox - qy * oy - qz * oz;
  real rx = qw * ox + qx * ow + qy * oz - qz * oy;
  real ry = qw * oy + qy * ow + qz * ox - qx * oz;
  real rz = qw * oz + qz * ow + qx * oy - qy * ox;
  // Quaternion::ToMatrix (Quaternion.h:46-72).
  M4 R = m4_identity();
  {
    real x = rx, y = ry, z = rz, w = rw;
    real *m = R.e;
    m[0] = 1.0f - 2.0f * (y * y + z * z);
    m[1] = 2.0f * (x * y + z * w);
    m[2] = 2.0f * (z * x - y * w);
    m[3] = 0.0f;
    m[4] = 2.0f * (x * y - z * w);
    m[5] = 1.0f - 2.0f * (z * z + x * x);
    m[6] = 2.0f * (y * z + x * w);
    m[7] = 0.0f;
    m[8] = 2.0f * (z * x + y * w);
    m[9] = 2.0f * (y * z - x * w);
    m[10] = 1.0f - 2.0f * (x * x + y * y);
    m[11] = 0.0f;
    m[12] = m[13] = m[14] = 0.0f;
    m[15] = 1.0f;
  }
  // Scene members (floats) from the PSART constructor (WaP_Tomo.cpp:251-286).
  real sid = (real)s->sid, sdd = (real)s->sdd;
  real tr0 = (real)(-s->oxyz[0]), tr2 = (real)(+s->oxyz[1]), tr1 = (real)(-s->oxyz[2]);
  double halfW = (s->det[0] - 1) * s->ds * 0.5f;
  double halfH = (s->det[1] - 1) * s->ds * 0.5f;
  // Scene::_calculateCamera (Scene.cpp:65-127).
  real zbase = -1 * sid;
  real nearp = sdd;
  real farp = (real)10000.0;
  // Scene::_calculateMatrix (Scene.cpp:163-189).
  M4 T = m4_identity();
  T.e[12] = tr0;
  T.e[13] = tr1;
  T.e[14] = zbase + tr2;
  M4 S = m4_identity();
  M4 view = m4_mul(m4_mul(T, S), R);
  M4 proj;
  proj.e[0] = (real)(nearp / halfW);
  proj.e[1] = proj.e[2] = proj.e[3] = 0.0f;
  proj.e[4] = 0.0f;
  proj.e[5] = (real)(nearp / halfH);
  proj.e[6] = proj.e[7] = proj.e[8] = proj.e[9] = 0.0f;
  proj.e[10] = -(farp + nearp) / (farp - nearp);
  proj.e[11] = -1.0f;
  proj.e[12] = proj.e[13] = 0.0f;
  proj.e[14] = -2.0f * farp * nearp / (farp - nearp);
  proj.e[15] = 0.0f;
  // TypicalRayProducer::SetVolSize / _calculateMatrix (TypicalRayProducer.cpp:118-232).
  real sp = (real)s->vs;
  real volsize[3] = {(s->vol[0] - 1) * sp, (s->vol[1] - 1) * sp, (s->vol[2] - 1) * sp};
  M4 Tv = m4_identity();
  Tv.e[12] = -volsize[0] * 0.5f;
  Tv.e[13] = -volsize[1] * 0.5f;
  Tv.e[14] = -volsize[2] * 0.5f;
  g.mv = m4_mul(view, Tv);
  M4 m2v = m4_identity();
  m2v.e[0] = 1.0f / sp;
  m2v.e[1] = m2v.e[2] = m2v.e[3] = m2v.e[4] = 0.0f;
  m2v.e[5] = 1.0f / sp;
  m2v.e[6] = m2v.e[7] = m2v.e[8] = m2v.e[9] = 0.0f;
  m2v.e[10] = 1.0f / sp;
  m2v.e[11] = m2v.e[12] = m2v.e[13] = m2v.e[14] = 0.0f;
  m2v.e[15] = 1.0f;
  g.m2v = m2v;
  g.v2m = m2v;
  m4_inverse(g.v2m);
  M4 v2p = m4_identity();
  v2p.e[0] = 0.5f * (s->det[0] - 1);
  v2p.e[1] = v2p.e[2] = v2p.e[3] = v2p.e[4] = 0.0f;
  v2p.e[5] = 0.5f * (s->det[1] - 1);
  v2p.e[6] = v2p.e[7] = v2p.e[8] = v2p.e[9] = 0.0f;
  v2p.e[10] = 0.5f;
  v2p.e[11] = 0.0f;
  v2p.e[12] = v2p.e[0];
  v2p.e[13] = v2p.e[5];
  v2p.e[14] = v2p.e[10];
  v2p.e[15] = 1.0f;
  M4 m2p = m4_mul(m4_mul(v2p, proj), g.mv);
  g.p2m = m2p;
  m4_inverse(g.p2m);
  g.eye[0] = g.p2m.e[8] / g.p2m.e[11];
  g.eye[1] = g.p2m.e[9] / g.p2m.e[11];
  g.eye[2] = g.p2m.e[10] / g.p2m.e[11];
  g.eye[3] = 1.0f;
  g.mvv2m = m4_mul(g.mv, g.v2m);
  return g;
}

// ---------------------------------------------------------------------------
// Forward projector
// ---------------------------------------------------------------------------
struct Vol {
  const real *d;
  int n[3];
  real at(int x, int y, int z) const {  // SingleScalarVolume.core.h:66-83
    x = mac_max(mac_min(x, n[0] - 1), 0);
    y = mac_max(mac_min(y, n[1] - 1), 0);
    z = mac_max(mac_min(z, n[2] - 1), 0);
    return d[x + (size_t)n[0] * (y + (size_t)n[1] * z)];
  }
};

struct Splat {
  real *contrib, *weight;
  real corr;
};

// T_VolumeAccess::GetScalarValue(Vector4) (SingleScalarVolume.core.h:99-202).
inline real sample_trilinear(const Vol &v, real p0, real p1, real p2, real &sumw, Splat *splat) {
  real pos[3] = {p0, p1, p2};
  for (int a = 0; a < 3; ++a) pos[a] = mac_max(mac_min(pos[a], (real)(v.n[a] - 1)), 0.0f);
  int ip[3] = {(int)pos[0], (int)pos[1], (int)pos[2]};
  if (splat) {
    real t0 = pos[0] - ip[0], t1 = pos[1] - ip[1], t2 = pos[2] - ip[2];
    real M0 = 1.0f - t0, M1 = 1.0f - t1, M2 = 1.0f - t2;
    real w[8] = {M0 * M1 * M2, t0 * M1 * M2, M0 * t1 * M2, t0 * t1 * M2,
                  M0 * M1 * t2, t0 * M1 * t2, M0 * t1 * t2, t0 * t1 * t2};
    // Taps past the last voxel carry weight 0 (pos is clamped to dim-1).
    for (int c = 0; c < 8; ++c) {
      int x = ip[0] + (c & 1), y = ip[1] + ((c >> 1) & 1), z = ip[2] + ((c >> 2) & 1);
      if (x >= v.n[0] || y >= v.n[1] || z >= v.n[2]) continue;
      size_t id = x + (size_t)v.n[0] * (y + (size_t)v.n[1] * z);
      splat->contrib[id] += splat->corr * w[c];
      splat->weight[id] += w[c];
    }
    return 0.0f;
  }
  real f2 = pos[0] - ip[0];
  real f1 = 1.0f - f2;
  sumw += 1.0f;
  real a = v.at(ip[0], ip[1], ip[2]) * f1 + v.at(ip[0] + 1, ip[1], ip[2]) * f2;
  real b = v.at(ip[0], ip[1] + 1, ip[2]) * f1 + v.at(ip[0] + 1, ip[1] + 1, ip[2]) * f2;
  real c = v.at(ip[0], ip[1], ip[2] + 1) * f1 + v.at(ip[0] + 1, ip[1], ip[2] + 1) * f2;
  real d = v.at(ip[0], ip[1] + 1, ip[2] + 1) * f1 + v.at(ip[0] + 1, ip[1] + 1, ip[2] + 1) * f2;
  f2 = pos[1] - ip[1];
  f1 = 1.0f - f2;
  a = a * f1 + b * f2;
  c = c * f1 + d * f2;
  f2 = pos[2] - ip[2];
  f1 = 1.0f - f2;
  return a * f1 + c * f2;
}

// CastingRay with block size == volume size (RayCaster.core.h:42-188,191-207).
real cast_ray(const Vol &v, const real vz[4], const real vu[4], real tnear, real tfar, real sd, real &sumw,
               Splat *splat) {
  real density = 0.0f;
  real t1 = tnear;
  real pos1[4];
  for (int a = 0; a < 4; ++a) pos1[a] = vz[a] + vu[a] * t1;
  real step[4];
  for (int a = 0; a < 4; ++a) step[a] = vu[a] * sd;
  real s1 = sample_trilinear(v, pos1[0], pos1[1], pos1[2], sumw, splat);
  density += s1 * sd;
  real tMax[3], tDelta[3] = {0.0f, 0.0f, 0.0f};
  for (int a = 0; a < 3; ++a) {
    int bs = v.n[a];
    int blk;
    if (vu[a] == 0) {
      blk = ((int)std::ceil(pos1[a] - 0.5f) - 1) / bs;
      tMax[a] = tfar;
    } else if (vu[a] < 0) {
      blk = ((int)std::ceil(pos1[a] - 0.5f) - 1) / bs;
      tMax[a] = (blk * bs + 0.5f - vz[a]) / vu[a];
      tDelta[a] = -(1 * bs) / vu[a];
    } else {
      blk = ((int)std::floor(pos1[a] - 0.5f)) / bs;
      tMax[a] = ((blk + 1) * bs + 0.5f - vz[a]) / vu[a];
      tDelta[a] = (1 * bs) / vu[a];
    }
  }
  while (t1 < tfar) {
    real tb = mac_min(mac_min(tMax[0], tMax[1]), tMax[2]);
    if (tb > tfar) tb = tfar;
    real t = std::ceil((t1 - tnear) / sd) * sd + tnear;
    real pos[4];
    for (int a = 0; a < 4; ++a) pos[a] = vz[a] + vu[a] * t;
    while (t < tb) {
      density += sample_trilinear(v, pos[0], pos[1], pos[2], sumw, splat) * sd;
      t += sd;
      for (int a = 0; a < 4; ++a) pos[a] += step[a];
    }
    if (tMax[0] < tMax[1]) {
      if (tMax[0] < tMax[2]) tMax[0] += tDelta[0];
      else tMax[2] += tDelta[2];
    } else {
      if (tMax[1] < tMax[2]) tMax[1] += tDelta[1];
      else tMax[2] += tDelta[2];
    }
    t1 = tb;
  }
  return density;
}

// ProduceRay (TypicalRayProducer.core.h:32-120).
inline void produce_ray(const ProjGeom &g, const int dims[3], real px, real py, real vz[4], real vu[4],
                        real &tnear, real &tfar) {
  real pin[4] = {px, py, 0.0f, 1.0f};
  real mp[4];
  m4_vec(g.p2m.e, pin, mp);
  real inv = 1.0f / mp[3];
  for (int a = 0; a < 4; ++a) mp[a] *= inv;
  real dir[4];
  for (int a = 0; a < 4; ++a) dir[a] = mp[a] - g.eye[a];
  real li = 1.0f / std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
  dir[0] *= li;
  dir[1] *= li;
  dir[2] *= li;
  m4_vec(g.m2v.e, g.eye, vz);
  m4_vec(g.m2v.e, dir, vu);
  real tmn[3], tmx[3];
  for (int a = 0; a < 3; ++a) {
    real lo = 0.0f, hi = (real)(dims[a] - 1);
    real t1 = (lo - vz[a]) / vu[a];
    real t2 = (hi - vz[a]) / vu[a];
    tmn[a] = mac_min(t1, t2);
    tmx[a] = mac_max(t1, t2);
  }
  tnear = mac_max(mac_max(tmn[0], tmn[1]), tmn[2]);
  tnear = mac_max(tnear, 0.0f);
  tfar = mac_min(mac_min(tmx[0], tmx[1]), tmx[2]);
}

// OpenMP threads for one call (t > 0; 0 keeps the current count), restored
// on return so that a call with its own count (advect's 4, as the reference's
// advect hard-codes) does not change the calls after it.
struct ThreadScope {
  int prev;
  explicit ThreadScope(int t) : prev(omp_get_max_threads()) {
    if (t > 0) omp_set_num_threads(t);
  }
  ~ThreadScope() { omp_set_num_threads(prev); }
  ThreadScope(const ThreadScope &) = delete;
  ThreadScope &operator=(const ThreadScope &) = delete;
};

// ---------------------------------------------------------------------------
// Bicubic backprojection helpers (WaP_Tomo.cpp:208-222, double arithmetic)
// ---------------------------------------------------------------------------
inline real cubic_interp(const real p[4], real x) {
  return p[1] + 0.5 * x * (p[2] - p[0] + x * (2.0 * p[0] - 5.0 * p[1] + 4.0 * p[2] - p[3] +
                                               x * (3.0 * (p[1] - p[2]) + p[3] - p[0])));
}

inline real bicubic_interp(real p[4][4], real x, real y) {
  real arr[4];
  arr[0] = cubic_interp(p[0], y);
  arr[1] = cubic_interp(p[1], y);
  arr[2] = cubic_interp(p[2], y);
  arr[3] = cubic_interp(p[3], y);
  return cubic_interp(arr, x);
}

// ---------------------------------------------------------------------------
// Advection (advection.h) with CImg's _cubic_atXYZ (CImg.h:13429-13524)
// ---------------------------------------------------------------------------
struct Img {
  const real *d;
  int n[3];
  real operator()(int x, int y, int z) const { return d[x + (size_t)n[0] * (y + (size_t)n[1] * z)]; }
};

inline real cimg_cut(real v, real lo, real hi) { return v < lo ? lo : (v > hi ? hi : v); }

inline real cub(real p, real c, real n, real a, real t) {
  return c + 0.5f * (t * (-p + n) + t * t * (2 * p - 5 * c + 4 * n - a) + t * t * t * (-p + 3 * c - 3 * n + a));
}

real cubic_atXYZ(const Img &I, real fx, real fy, real fz) {
  const real nfx = cimg_cut(fx, 0, I.n[0] - 1), nfy = cimg_cut(fy, 0, I.n[1] - 1), nfz = cimg_cut(fz, 0, I.n[2] - 1);
  const int x = (int)nfx, y = (int)nfy, z = (int)nfz;
  const real dx = nfx - x, dy = nfy - y, dz = nfz - z;
  const int px = x - 1 < 0 ? 0 : x - 1, nx = dx > 0 ? x + 1 : x, ax = x + 2 >= I.n[0] ? I.n[0] - 1 : x + 2;
  const int py = y - 1 < 0 ? 0 : y - 1, ny = dy > 0 ? y + 1 : y, ay = y + 2 >= I.n[1] ? I.n[1] - 1 : y + 2;
  const int pz = z - 1 < 0 ? 0 : z - 1, nz = dz > 0 ? z + 1 : z, az = z + 2 >= I.n[2] ? I.n[2] - 1 : z + 2;
  const int xs[4] = {px, x, nx, ax}, ys[4] = {py, y, ny, ay}, zs[4] = {pz, z, nz, az};
  real planes[4];
  for (int kz = 0; kz < 4; ++kz) {
    real rows[4];
    for (int ky = 0; ky < 4; ++ky)
      rows[ky] = cub(I(xs[0], ys[ky], zs[kz]), I(xs[1], ys[ky], zs[kz]), I(xs[2], ys[ky], zs[kz]),
                     I(xs[3], ys[ky], zs[kz]), dx);
    planes[kz] = cub(rows[0], rows[1], rows[2], rows[3], dy);
  }
  return cub(planes[0], planes[1], planes[2], planes[3], dz);
}

// advection::sample_image (advection.h:49-88).
real sample_image(const int dims[3], const real aabb[6], const Img &I, const real p[3]) {
  real g[3];
  for (int a = 0; a < 3; ++a)
    g[a] = (real)((double)((real)dims[a] * (p[a] - aabb[2 * a]) / (aabb[2 * a + 1] - aabb[2 * a])) - 0.5);
  for (int a = 0; a < 3; ++a) g[a] = std_max(1.0f, std_min((real)(dims[a] - 2), g[a]));
  int ix = (int)g[0], iy = (int)g[1], iz = (int)g[2];
  real mn = I(ix, iy, iz), mx = mn;
  const int o[7][3] = {{1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  for (int q = 0; q < 7; ++q) {
    real v = I(ix + o[q][0], iy + o[q][1], iz + o[q][2]);
    mn = std_min(mn, v);
    mx = std_max(mx, v);
  }
  return std_max(mn, std_min(mx, cubic_atXYZ(I, g[0], g[1], g[2])));
}

void sample_velocity(const int dims[3], const real aabb[6], const real *vel, const real p[3], real v[3]) {
  size_t nv = (size_t)dims[0] * dims[1] * dims[2];
  for (int c = 0; c < 3; ++c) {
    Img I{vel + c * nv, {dims[0], dims[1], dims[2]}};
    v[c] = sample_image(dims, aabb, I, p);
  }
}

}  // namespace

extern "C" {

// VolumeData::ReadStructuredFile (VolumeData.cpp:133-210): nf, timeunit, windows.
int orc_level_frames(int nframes_cli, int nproj, int level, int *start, int *end, real *ftime, real *tunit) {
  int factor = 1 << level;
  int nf = std::min(nframes_cli * factor, 130);
  real timeunit = (real)((real)nproj / (real)nf);
  real baseNo = 3;
  for (int i = 0; i < nf; ++i) {
    real t = timeunit * i;
    if (ftime) ftime[i] = t;
    if (start) start[i] = std::max(0, (int)(t - baseNo));
    if (end) end[i] = std::min((int)(t + baseNo), nproj - 1);
  }
  if (tunit) *tunit = timeunit;
  return nf;
}

real orc_sample_distance(double vs) {
  // PSART::SetData (WaP_Tomo.cpp:380): sqrt of the real sum of squares / 2.
  real sp = (real)vs;
  return std::sqrt(sp * sp + sp * sp + sp * sp) / 2;
}

void orc_geometry(const orc_scan *s, double angle_deg, real p2m[16], real m2v[16], real mv[16], real v2m[16],
                  real eye[4]) {
  ProjGeom g = make_geometry(s, angle_deg);
  std::memcpy(p2m, g.p2m.e, 16 * sizeof(real));
  std::memcpy(m2v, g.m2v.e, 16 * sizeof(real));
  std::memcpy(mv, g.mv.e, 16 * sizeof(real));
  std::memcpy(v2m, g.v2m.e, 16 * sizeof(real));
  std::memcpy(eye, g.eye, 4 * sizeof(real));
}

// GenerateImage_MT (TypicalRayProducer.core.h:123-225).
void orc_forward(const orc_scan *s, double angle_deg, const real *vol, real *img, real *len, real *weight) {
  ThreadScope threads_scope(s->threads);
  ProjGeom g = make_geometry(s, angle_deg);
  const int W = s->det[0], H = s->det[1];
  const real sd = orc_sample_distance(s->vs);
  Vol v{vol, {s->vol[0], s->vol[1], s->vol[2]}};
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      int k = i + j * W;
      real vz[4], vu[4], tn, tf;
      produce_ray(g, s->vol, (real)i, (real)j, vz, vu, tn, tf);
      real sumw = 0.0f;
      double value = 0.0f;
      len[k] = 0.0f;
      if (tn < tf) {
        len[k] = tf - tn;
        value = cast_ray(v, vz, vu, tn, tf, sd, sumw, nullptr);
      }
      weight[k] = sumw;
      img[k] = (real)value;
    }
}

// Back-projection mode of the same traversal, single-threaded (the
// reference's += on shared voxels races under OpenMP).
void orc_ray_backproject(const orc_scan *s, double angle_deg, const real *corr, real *contrib, real *weight) {
  ProjGeom g = make_geometry(s, angle_deg);
  const int W = s->det[0], H = s->det[1];
  const real sd = orc_sample_distance(s->vs);
  size_t nv = (size_t)s->vol[0] * s->vol[1] * s->vol[2];
  std::memset(contrib, 0, nv * sizeof(real));
  std::memset(weight, 0, nv * sizeof(real));
  Vol v{nullptr, {s->vol[0], s->vol[1], s->vol[2]}};
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      real vz[4], vu[4], tn, tf;
      produce_ray(g, s->vol, (real)i, (real)j, vz, vu, tn, tf);
      real sumw = 0.0f;
      if (tn < tf) {
        Splat sp{contrib, weight, corr[i + j * W]};
        cast_ray(v, vz, vu, tn, tf, sd, sumw, &sp);
      }
    }
}

// WaP_Tomo.cpp:1530-1555: c = (F p - F Ax - y)/(F len + 1), y += alpha c, F = 1.
void orc_correction(int n, const real *p, const real *ax, const real *len, real *dual, double alpha, real *c) {
  const real F = std::sqrt(2 * (1.0f / 2));
  for (int k = 0; k < n; ++k) {
    real y = dual ? dual[k] : 0.0f;
    c[k] = (real)(F * p[k] - F * ax[k] - y) / (real)(F * len[k] + 1.0f);
    if (dual) dual[k] += alpha * c[k];
  }
}

void orc_bp_voxel(const orc_scan *s, double angle_deg, const real *corr, const int box[6], int mode, real *vol) {
  ThreadScope threads_scope(s->threads);
  ProjGeom g = make_geometry(s, angle_deg);
  const int W = s->det[0], H = s->det[1];
  const int *d = s->vol;
  const double halfW = (W - 1) * s->ds * 0.5f, halfH = (H - 1) * s->ds * 0.5f;
  const real sdd = (real)s->sdd;
  const double ds = s->ds;
  const double alpha = s->alpha;
  const real gmax = s->gmax;
  const int iminY = W;
#pragma omp parallel for
  for (int z = box[4]; z < box[5]; ++z)
    for (int y = box[2]; y < box[3]; ++y)
      for (int x = box[0]; x < box[1]; ++x) {
        size_t pos = x + (size_t)d[0] * (y + (size_t)d[1] * z);
        real vec[4] = {(real)x, (real)y, (real)z, 1.0f};
        real det[4];
        m4_vec(g.mvv2m.e, vec, det);
        real _px = halfW - (det[0] / det[2]) * sdd;
        real _py = halfH - (det[1] / det[2]) * sdd;
        _px = _px / ds;
        _py = _py / ds;
        int px = (int)_px, py = (int)_py;
        real dx = _px - px, dy = _py - py;
        if (px < 2 || px >= W - 2 || py < 2 || py >= H - 2) continue;
        const real *pC = corr + py * W + px;
        real pimg[4][4] = {{pC[-1 - iminY], pC[-1], pC[-1 + iminY], pC[-1 + 2 * iminY]},
                            {pC[-iminY], pC[0], pC[iminY], pC[2 * iminY]},
                            {pC[1 - iminY], pC[1], pC[1 + iminY], pC[1 + 2 * iminY]},
                            {pC[2 - iminY], pC[2], pC[2 + iminY], pC[2 + 2 * iminY]}};
        real gv = bicubic_interp(pimg, dx, dy);
        if (mode == 0) {
          vol[pos] += alpha * gv;
          vol[pos] = mac_max(mac_min(gmax, vol[pos]), 0);
        } else {
          vol[pos] += gv;
        }
      }
}

void orc_advect(const int dims[3], const real aabb[6], const real *vel, const real *src, int nc, real dt,
                real *out, int threads) {
  ThreadScope threads_scope(threads);
  const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
  const real tdt = -dt;  // advect calls trace(..., -dt)
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < dims[2]; ++k)
    for (int j = 0; j < dims[1]; ++j)
      for (int i = 0; i < dims[0]; ++i) {
        const int gi[3] = {i, j, k};
        real p[3];
        for (int a = 0; a < 3; ++a) {
          real gf = (real)gi[a];
          p[a] = (real)(aabb[2 * a] + (gf + 0.5) * (aabb[2 * a + 1] - aabb[2 * a]) / (real)dims[a]);
        }
        // trace (advection.h:101-115)
        real v[3], p2[3], p0[3], q[3];
        sample_velocity(dims, aabb, vel, p, v);
        for (int a = 0; a < 3; ++a) p2[a] = p[a] + tdt * v[a];
        sample_velocity(dims, aabb, vel, p2, v);
        for (int a = 0; a < 3; ++a) p0[a] = p2[a] - tdt * v[a];
        for (int a = 0; a < 3; ++a) q[a] = p2[a] + (real)(0.5 * (real)(p[a] - p0[a]));
        for (int c = 0; c < nc; ++c) {
          Img I{src + c * nv, {dims[0], dims[1], dims[2]}};
          out[c * nv + i + (size_t)dims[0] * (j + (size_t)dims[1] * k)] = sample_image(dims, aabb, I, q);
        }
      }
}

// CImg::deriche order 0 with Neumann boundaries (CImg.h:32917-33010) applied
// along x, then y, then z (CImg::blur, CImg.h:33249-33262).
void orc_blur(const int dims[3], int nc, real sigma, const real *src, real *out) {
  const size_t nv = (size_t)dims[0] * dims[1] * dims[2];
  std::memcpy(out, src, nv * nc * sizeof(real));
  const real nsigma = sigma >= 0 ? sigma : 0.0f;
  if (nsigma < 0.1f) return;
  const real nnsigma = nsigma < 0.1f ? 0.1f : nsigma, alpha = 1.695f / nnsigma, ema = (real)std::exp(-alpha),
              ema2 = (real)std::exp(-2 * alpha), b1 = -2 * ema, b2 = ema2;
  const real k = (1 - ema) * (1 - ema) / (1 + 2 * alpha * ema - ema2);
  const real a0 = k, a1 = k * (alpha - 1) * ema, a2 = k * (alpha + 1) * ema, a3 = -k * ema2;
  const real coefp = (a0 + a1) / (1 + b1 + b2), coefn = (a2 + a3) / (1 + b1 + b2);
  const size_t stride[3] = {1, (size_t)dims[0], (size_t)dims[0] * dims[1]};
  for (int axis = 0; axis < 3; ++axis) {
    const int N = dims[axis];
    if (N <= 1) continue;
    const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
    const size_t off = stride[axis];
#pragma omp parallel for collapse(2)
    for (int c = 0; c < nc; ++c)
      for (int u = 0; u < dims[o2]; ++u)
        for (int w = 0; w < dims[o1]; ++w) {
          real *ptr = out + c * nv + w * stride[o1] + u * stride[o2];
          std::vector<real> Y(N);
          real yb = 0, yp = 0, xp = 0;
          xp = ptr[0];
          yb = yp = coefp * xp;
          for (int m = 0; m < N; ++m) {
            const real xc = ptr[m * off];
            const real yc = Y[m] = a0 * xc + a1 * xp - b1 * yp - b2 * yb;
            xp = xc;
            yb = yp;
            yp = yc;
          }
          real xn = ptr[(N - 1) * off], xa = xn, yn = coefn * xn, ya = yn;
          for (int n = N - 1; n >= 0; --n) {
            const real xc = ptr[n * off];
            const real yc = a2 * xn + a3 * xa - b1 * yn - b2 * ya;
            xa = xn;
            xn = xc;
            ya = yn;
            yn = yc;
            ptr[n * off] = Y[n] + yc;
          }
        }
  }
}

// CImg::get_resize(sx,sy,sz,sc, 5, 0): per axis, moving average when
// shrinking (CImg.h:28135-28213) or the double-precision cubic when growing
// (CImg.h:28432-28610), axes in the order x, y, z.
void orc_resize(const int dims[3], int nc, const real *src, const int odims[3], real *out) {
  std::vector<real> cur(src, src + (size_t)dims[0] * dims[1] * dims[2] * nc);
  int cd[3] = {dims[0], dims[1], dims[2]};
  for (int axis = 0; axis < 3; ++axis) {
    const int Sin = cd[axis], Sout = odims[axis];
    if (Sin == Sout) continue;
    int nd[3] = {cd[0], cd[1], cd[2]};
    nd[axis] = Sout;
    const size_t in_stride[3] = {1, (size_t)cd[0], (size_t)cd[0] * cd[1]};
    const size_t out_stride[3] = {1, (size_t)nd[0], (size_t)nd[0] * nd[1]};
    const size_t in_nv = (size_t)cd[0] * cd[1] * cd[2], out_nv = (size_t)nd[0] * nd[1] * nd[2];
    std::vector<real> nxt(out_nv * nc, 0.0f);
    const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
    if (Sin == 1) {
      // nearest-neighbour replication (CImg falls back to interpolation 1)
      for (int ch = 0; ch < nc; ++ch)
        for (int u = 0; u < cd[o2]; ++u)
          for (int w = 0; w < cd[o1]; ++w)
            for (int t = 0; t < Sout; ++t)
              nxt[ch * out_nv + w * out_stride[o1] + u * out_stride[o2] + t * out_stride[axis]] =
                  cur[ch * in_nv + w * in_stride[o1] + u * in_stride[o2]];
    } else if (Sin > Sout) {
      // moving average: accumulate src*d per output cell, divide by Sin.
      std::vector<std::vector<std::pair<int, unsigned>>> taps(Sout);
      for (unsigned a = Sin * Sout, b = Sin, c = Sout, s = 0, t = 0; a;) {
        const unsigned d = std::min(b, c);
        a -= d;
        b -= d;
        c -= d;
        taps[t].push_back({(int)s, d});
        if (!b) {
          ++t;
          b = Sin;
        }
        if (!c) {
          ++s;
          c = Sout;
        }
      }
      for (int ch = 0; ch < nc; ++ch)
        for (int u = 0; u < cd[o2]; ++u)
          for (int w = 0; w < cd[o1]; ++w)
            for (int t = 0; t < Sout; ++t) {
              real acc = 0.0f;
              for (auto &tp : taps[t])
                acc += cur[ch * in_nv + w * in_stride[o1] + u * in_stride[o2] + tp.first * in_stride[axis]] *
                       (real)tp.second;
              acc /= (real)(unsigned)Sin;
              nxt[ch * out_nv + w * out_stride[o1] + u * out_stride[o2] + t * out_stride[axis]] = acc;
            }
    } else {
      const double f = Sout > 1 ? (Sin - 1.0) / (Sout - 1) : 0;
      std::vector<unsigned> base(Sout);
      std::vector<double> frac(Sout);
      double curr = 0, old = 0;
      unsigned idx = 0;
      for (int x = 0; x < Sout; ++x) {
        frac[x] = curr - (unsigned)curr;
        base[x] = idx;
        old = curr;
        curr = std::min(Sin - 1.0, curr + f);
        idx += (unsigned)curr - (unsigned)old;
      }
      const double vmin = -3.4028234663852886e38, vmax = 3.4028234663852886e38;
      for (int ch = 0; ch < nc; ++ch)
        for (int u = 0; u < cd[o2]; ++u)
          for (int w = 0; w < cd[o1]; ++w) {
            const real *line = cur.data() + ch * in_nv + w * in_stride[o1] + u * in_stride[o2];
            const size_t st = in_stride[axis];
            for (int x = 0; x < Sout; ++x) {
              const int i = (int)base[x];
              const double t = frac[x];
              const double val1 = line[i * st];
              const double val0 = i > 0 ? (double)line[(i - 1) * st] : val1;
              const double val2 = i <= Sin - 2 ? (double)line[(i + 1) * st] : val1;
              const double val3 = i < Sin - 2 ? (double)line[(i + 2) * st] : val2;
              const double val = val1 + 0.5f * (t * (-val0 + val2) + t * t * (2 * val0 - 5 * val1 + 4 * val2 - val3) +
                                                t * t * t * (-val0 + 3 * val1 - 3 * val2 + val3));
              nxt[ch * out_nv + w * out_stride[o1] + u * out_stride[o2] + x * out_stride[axis]] =
                  (real)(val < vmin ? vmin : val > vmax ? vmax : val);
            }
          }
    }
    cur.swap(nxt);
    cd[axis] = Sout;
  }
  std::memcpy(out, cur.data(), cur.size() * sizeof(real));
}

void orc_gradient(const int dims[3], const real *src, real *gx, real *gy, real *gz) {
  Img I{src, {dims[0], dims[1], dims[2]}};
  for (int z = 0; z < dims[2]; ++z)
    for (int y = 0; y < dims[1]; ++y)
      for (int x = 0; x < dims[0]; ++x) {
        size_t id = x + (size_t)dims[0] * (y + (size_t)dims[1] * z);
        int xp = x > 0 ? x - 1 : x, xn = x < dims[0] - 1 ? x + 1 : x;
        int yp = y > 0 ? y - 1 : y, yn = y < dims[1] - 1 ? y + 1 : y;
        int zp = z > 0 ? z - 1 : z, zn = z < dims[2] - 1 ? z + 1 : z;
        gx[id] = (I(xn, y, z) - I(xp, y, z)) / 2;
        gy[id] = (I(x, yn, z) - I(x, yp, z)) / 2;
        gz[id] = (I(x, y, zn) - I(x, y, zp)) / 2;
      }
}

}  // extern "C"

namespace {

// tools.cpp:247-313 finite differences on a volume.
struct Grid {
  int n[3];
  size_t id(int i, int j, int k) const { return i + (size_t)n[0] * (j + (size_t)n[1] * k); }
};

inline real dxp3(const real *d, const Grid &g, int i, int j, int k) {
  return i < g.n[0] - 1 ? d[g.id(i + 1, j, k)] - d[g.id(i, j, k)] : 0.0f;
}
inline real dyp3(const real *d, const Grid &g, int i, int j, int k) {
  return j < g.n[1] - 1 ? d[g.id(i, j + 1, k)] - d[g.id(i, j, k)] : 0.0f;
}
inline real dzp3(const real *d, const Grid &g, int i, int j, int k) {
  return k < g.n[2] - 1 ? d[g.id(i, j, k + 1)] - d[g.id(i, j, k)] : 0.0f;
}
inline real dxm3(const real *d, const Grid &g, int i, int j, int k) {
  if (i > 0 && i < g.n[0] - 1) return d[g.id(i, j, k)] - d[g.id(i - 1, j, k)];
  if (i == 0) return d[g.id(i, j, k)];
  return -d[g.id(i - 1, j, k)];
}
inline real dym3(const real *d, const Grid &g, int i, int j, int k) {
  if (j > 0 && j < g.n[1] - 1) return d[g.id(i, j, k)] - d[g.id(i, j - 1, k)];
  if (j == 0) return d[g.id(i, j, k)];
  return -d[g.id(i, j - 1, k)];
}
inline real dzm3(const real *d, const Grid &g, int i, int j, int k) {
  if (k > 0 && k < g.n[2] - 1) return d[g.id(i, j, k)] - d[g.id(i, j, k - 1)];
  if (k == 0) return d[g.id(i, j, k)];
  return -d[g.id(i, j, k - 1)];
}
inline real my_abs(real x) { return x > 0 ? x : -x; }

}  // namespace

static double g_last_pd_seconds = 0.0;

extern "C" {

double orc_last_pd_seconds() { return g_last_pd_seconds; }

int orc_flow_level(const int dims[3], const real *I1, const real *I2, real *V, real *Y1, real *Y2, real *Y3,
                   real *Y4, real tol, real lambda, int max_iters, int nwarps, const real aabb[6],
                   const int roi6[6], int deterministic, int *iters_out) {
  const Grid g{{dims[0], dims[1], dims[2]}};
  const int nPx = dims[0] * dims[1] * dims[2];
  const size_t n = (size_t)nPx;
  std::vector<real> v[3], vOld[3], y[9], yOld[9], Kty[3], KtyOld[3], Kx[9], KxOld[9];
  std::vector<real> y4(n), y4Old(n), Kx4(n, 0.0f), Kx4Old(n, 0.0f), ux(n, 0.0f), uy(n, 0.0f), uz(n, 0.0f),
      ut(n, 0.0f), tau[3], sigma2(n);
  for (int c = 0; c < 3; ++c) {
    v[c].assign(V + c * n, V + (c + 1) * n);
    vOld[c].assign(n, 0.0f);
    Kty[c].assign(n, 0.0f);
    KtyOld[c].assign(n, 0.0f);
    tau[c].assign(n, 0.0f);
  }
  const real *Ys[3] = {Y1, Y2, Y3};
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) {
      y[3 * a + c].assign(Ys[a] + c * n, Ys[a] + (c + 1) * n);
      yOld[3 * a + c].assign(n, 0.0f);
      Kx[3 * a + c].assign(n, 0.0f);
      KxOld[3 * a + c].assign(n, 0.0f);
    }
  y4.assign(Y4, Y4 + n);
  const real sigma1 = std::min(1.0f / 3.0f, std::min(1.0f / 3.0f, 1.0f / 3.0f));
  const int *roi = roi6;
  const int x0 = roi[0], x1 = dims[0] - roi[1], y0 = roi[2], y1 = dims[1] - roi[3], z0 = roi[4], z1 = dims[2] - roi[5];
  real p = 0.0f, d = 0.0f;
  int total = 0;
  double pd_seconds = 0.0;
  std::vector<real> Vimg(3 * n), warp(n), gx(n), gy(n), gz(n);
  for (int w = 0; w < nwarps; ++w) {
    // _inputV holds v inside the ROI (written by the primal) and the input outside.
    for (int c = 0; c < 3; ++c) std::memcpy(Vimg.data() + c * n, V + c * n, n * sizeof(real));
    orc_advect(dims, aabb, Vimg.data(), I2, 1, -1.0f, warp.data(), 0);
    orc_gradient(dims, warp.data(), gx.data(), gy.data(), gz.data());
#pragma omp parallel for
    for (int k = z0; k < z1; ++k)
      for (int j = y0; j < y1; ++j)
        for (int i = x0; i < x1; ++i) {
          size_t t = g.id(i, j, k);
          ux[t] = gx[t];
          uy[t] = gy[t];
          uz[t] = gz[t];
          ut[t] = warp[t] - I1[t] - ux[t] * v[0][t] - uy[t] * v[1][t] - uz[t] * v[2][t];
        }
#pragma omp parallel for
    for (int i = 0; i < nPx; ++i) {
      tau[0][i] = 4.0f / 1.0f + my_abs(ux[i]);
      tau[1][i] = 4.0f / 1.0f + my_abs(uy[i]);
      tau[2][i] = 4.0f / 1.0f + my_abs(uz[i]);
      sigma2[i] = std::abs(ux[i]) + std::abs(uy[i]) + std::abs(uz[i]);
      tau[0][i] = 1.0f / tau[0][i];
      tau[1][i] = 1.0f / tau[1][i];
      tau[2][i] = 1.0f / tau[2][i];
      sigma2[i] = 1.0f / sigma2[i];
    }
    int it = 0;
    real err = 1.0f;
    const real *uu[3] = {ux.data(), uy.data(), uz.data()};
    const double t_pd = omp_get_wtime();
    while (err > tol && it <= max_iters) {
      ++it;
      const bool res = (it % 50 == 0);
      if (res) {
        p = 0.0f;
        d = 0.0f;
      }
      // primal (optical_flow.h:489-553)
      auto primal = [&](int i, int j, int k, real &acc) {
        size_t t = g.id(i, j, k);
        if (res)
          for (int c = 0; c < 3; ++c) {
            vOld[c][t] = v[c][t];
            KtyOld[c][t] = Kty[c][t];
          }
        for (int c = 0; c < 3; ++c) {
          Kty[c][t] = -1.0f * dxm3(y[3 * c].data(), g, i, j, k) - 1.0f * dym3(y[3 * c + 1].data(), g, i, j, k) -
                      1.0f * dzm3(y[3 * c + 2].data(), g, i, j, k) + uu[c][t] * y4[t];
        }
        for (int c = 0; c < 3; ++c) {
          v[c][t] -= tau[c][t] * Kty[c][t];
          V[c * n + t] = v[c][t];
        }
        if (res)
          acc += std::abs((vOld[0][t] - v[0][t]) / tau[0][t] - KtyOld[0][t] + Kty[0][t]) +
                 std::abs((vOld[1][t] - v[1][t]) / tau[1][t] - KtyOld[1][t] + Kty[1][t]) +
                 std::abs((vOld[2][t] - v[2][t]) / tau[2][t] - KtyOld[2][t] + Kty[2][t]);
      };
      if (deterministic) {
        for (int k = z0; k < z1; ++k)
          for (int j = y0; j < y1; ++j)
            for (int i = x0; i < x1; ++i) primal(i, j, k, p);
      } else {
        real pp = 0.0f;
#pragma omp parallel for reduction(+ : pp)
        for (int k = z0; k < z1; ++k)
          for (int j = y0; j < y1; ++j)
            for (int i = x0; i < x1; ++i) primal(i, j, k, pp);
        p += pp;
      }
      // dual (optical_flow.h:567-813), norm != 4 branch
      // over every voxel in index order (the reference's flat tmpIndex loop with
      // its i/j/k tables; nested loops here give the same order without a
      // division per voxel)
      auto dual = [&](int i, int j, int k, real &acc) {
        const size_t t = g.id(i, j, k);
        if (res) {
          for (int q = 0; q < 9; ++q) yOld[q][t] = y[q][t];
          y4Old[t] = y4[t];
        }
        for (int q = 0; q < 9; ++q) KxOld[q][t] = Kx[q][t];
        Kx4Old[t] = Kx4[t];
        for (int c = 0; c < 3; ++c) {
          Kx[3 * c][t] = 1.0f * dxp3(v[c].data(), g, i, j, k);
          Kx[3 * c + 1][t] = 1.0f * dyp3(v[c].data(), g, i, j, k);
          Kx[3 * c + 2][t] = 1.0f * dzp3(v[c].data(), g, i, j, k);
        }
        Kx4[t] = ux[t] * v[0][t] + uy[t] * v[1][t] + uz[t] * v[2][t];
        for (int q = 0; q < 9; ++q) {
          real yt = y[q][t] + sigma1 * (Kx[q][t] + Kx[q][t] - KxOld[q][t]);
          y[q][t] = yt * lambda / (lambda + 2 * sigma1);
        }
        y4[t] = std_max(-1.0f, std_min(1.0f, y4[t] + sigma2[t] * (Kx4[t] + Kx4[t] - Kx4Old[t] + ut[t])));
        if (res) {
          real s = 0.0f;
          for (int q = 0; q < 9; ++q) {
            real term = std::abs((yOld[q][t] - y[q][t]) / sigma1 - KxOld[q][t] + Kx[q][t]);
            s = (q == 0) ? term : s + term;
          }
          s = s + std::abs((y4Old[t] - y4[t]) / sigma2[t] - Kx4Old[t] + Kx4[t]);
          acc += s;
        }
      };
      if (deterministic) {
        for (int k = 0; k < dims[2]; ++k)
          for (int j = 0; j < dims[1]; ++j)
            for (int i = 0; i < dims[0]; ++i) dual(i, j, k, d);
      } else {
        real dd = 0.0f;
#pragma omp parallel for reduction(+ : dd)
        for (int k = 0; k < dims[2]; ++k)
          for (int j = 0; j < dims[1]; ++j)
            for (int i = 0; i < dims[0]; ++i) dual(i, j, k, dd);
        d += dd;
      }
      if (res) err = (d * d + p * p) / (real)nPx;
    }
    pd_seconds += omp_get_wtime() - t_pd;
    if (iters_out) iters_out[w] = it;
    total += it;
  }
  g_last_pd_seconds = pd_seconds;
  // write back (optical_flow.h:840-877): ROI only
  for (int k = z0; k < z1; ++k)
    for (int j = y0; j < y1; ++j)
      for (int i = x0; i < x1; ++i) {
        size_t t = g.id(i, j, k);
        for (int c = 0; c < 3; ++c) {
          Y1[c * n + t] = y[c][t];
          Y2[c * n + t] = y[3 + c][t];
          Y3[c * n + t] = y[6 + c][t];
          V[c * n + t] = v[c][t];
        }
        Y4[t] = y4[t];
      }
  return total;
}

int orc_flow_multiscale(const int dims[3], const real *I1, const real *I2, const real *V0, real tol,
                        real lambda, int max_iters, int nwarps, real eta, real sigma, int scales,
                        const int cut6[6], int deterministic, real *Vout) {
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<real> b1(n), b2(n);
  orc_blur(dims, 1, sigma, I1, b1.data());
  orc_blur(dims, 1, sigma, I2, b2.data());
  struct Lvl {
    int d[3];
    std::vector<real> i1, i2, v, y1, y2, y3, y4;
  };
  std::vector<Lvl> L(scales);
  real t_eta = 1.0f;
  for (int s = 0; s < scales; ++s) {
    Lvl &l = L[scales - 1 - s];  // reversed: coarse first
    l.d[0] = (int)(dims[0] * t_eta);
    l.d[1] = (int)(dims[1] * t_eta);
    l.d[2] = (int)(dims[2] * t_eta);
    size_t m = (size_t)l.d[0] * l.d[1] * l.d[2];
    l.i1.resize(m);
    l.i2.resize(m);
    l.v.resize(3 * m);
    orc_resize(dims, 1, b1.data(), l.d, l.i1.data());
    orc_resize(dims, 1, b2.data(), l.d, l.i2.data());
    orc_resize(dims, 3, V0, l.d, l.v.data());
    l.y1.assign(3 * m, 0.0f);  // resize of a zero field is zero
    l.y2.assign(3 * m, 0.0f);
    l.y3.assign(3 * m, 0.0f);
    l.y4.assign(m, 0.0f);
    t_eta = t_eta * eta;
  }
  int total = 0;
  const real aabb[6] = {0, (real)dims[0], 0, (real)dims[1], 0, (real)dims[2]};
  for (int s = 0; s < scales; ++s) {
    Lvl &l = L[s];
    int roi[6];
    for (int i = 0; i < 6; ++i) {
      int a = i / 2;
      roi[i] = (real)cut6[i] * ((real)l.d[a] / (real)dims[a]);
    }
    total += orc_flow_level(l.d, l.i1.data(), l.i2.data(), l.v.data(), l.y1.data(), l.y2.data(), l.y3.data(),
                            l.y4.data(), tol, lambda, max_iters, nwarps, aabb, roi, deterministic, nullptr);
    if (s < scales - 1) {
      Lvl &nx = L[s + 1];
      orc_resize(l.d, 3, l.v.data(), nx.d, nx.v.data());
      orc_resize(l.d, 3, l.y1.data(), nx.d, nx.y1.data());
      orc_resize(l.d, 3, l.y2.data(), nx.d, nx.y2.data());
      orc_resize(l.d, 3, l.y3.data(), nx.d, nx.y3.data());
      orc_resize(l.d, 1, l.y4.data(), nx.d, nx.y4.data());
    }
  }
  std::memcpy(Vout, L[scales - 1].v.data(), 3 * n * sizeof(real));
  return total;
}

// SART_Proximal_Operator (WaP_Tomo.cpp:1424-1678).
void orc_sart_prox(const orc_scan *s, const double *angles, const real *projs, int pstart, int pend, int nb_sart,
                   const int box[6], real *vol, real *dual_rows) {
  const int W = s->det[0], H = s->det[1];
  const size_t np = (size_t)W * H;
  const size_t nv = (size_t)s->vol[0] * s->vol[1] * s->vol[2];
  std::memset(dual_rows, 0, sizeof(real) * np * s->nproj);
  std::vector<real> img(np), len(np), wt(np), c(np);
  const int num = pend - pstart + 1;
  std::vector<int> order(num);
  for (int i = 0; i < num; ++i) order[i] = (i % 2 == 0) ? pstart + i / 2 : pend - i / 2;
  for (int iter = 1; iter <= nb_sart; ++iter)
    for (int q = 0; q < num; ++q) {
      const int pid = order[q];
      orc_forward(s, angles[pid], vol, img.data(), len.data(), wt.data());
      orc_correction((int)np, projs + np * pid, img.data(), len.data(), dual_rows + np * pid, s->alpha, c.data());
      orc_bp_voxel(s, angles[pid], c.data(), box, 0, vol);
    }
  for (size_t i = 0; i < nv; ++i) vol[i] = mac_max(vol[i] * 1.0f, 0.0f);
}

// The SART proximal operator with the ray-driven matched backprojection
// (the reference's back-projection mode of the ray caster,
// SingleScalarVolume.core.h:85-96,149-199, selected by --bp Raybased,
// TypicalRayProducer.cpp:42-45): the correction is splatted into per-voxel
// contribution and weight sums, and the volume takes alpha * contribution /
// weight where the weight is positive (column-sum normalisation), clamped to
// [0, G_Max], over the box.  The reference never consumes its sums, so this
// update is the one the library defines for the mode.
void orc_sart_prox_ray(const orc_scan *s, const double *angles, const real *projs, int pstart, int pend, int nb_sart,
                       const int box[6], real *vol, real *dual_rows) {
  const int W = s->det[0], H = s->det[1];
  const size_t np = (size_t)W * H;
  const int *d = s->vol;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  std::memset(dual_rows, 0, sizeof(real) * np * s->nproj);
  std::vector<real> img(np), len(np), wt(np), c(np), contrib(nv), weight(nv);
  const int num = pend - pstart + 1;
  const real a = (real)(float)s->alpha, gmax = s->gmax;
  for (int iter = 1; iter <= nb_sart; ++iter)
    for (int q = 0; q < num; ++q) {
      const int pid = (q % 2 == 0) ? pstart + q / 2 : pend - q / 2;
      orc_forward(s, angles[pid], vol, img.data(), len.data(), wt.data());
      orc_correction((int)np, projs + np * pid, img.data(), len.data(), dual_rows + np * pid, s->alpha, c.data());
      std::fill(contrib.begin(), contrib.end(), (real)0);
      std::fill(weight.begin(), weight.end(), (real)0);
      orc_ray_backproject(s, angles[pid], c.data(), contrib.data(), weight.data());
      for (int k = box[4]; k < box[5]; ++k)
        for (int j = box[2]; j < box[3]; ++j)
          for (int i = box[0]; i < box[1]; ++i) {
            const size_t t = i + (size_t)d[0] * (j + (size_t)d[1] * k);
            const real w = weight[t];
            if (!(w > (real)0)) continue;
            real v = vol[t] + a * (contrib[t] / w);
            vol[t] = v < (real)0 ? (real)0 : (v > gmax ? gmax : v);
          }
    }
  for (size_t i = 0; i < nv; ++i) vol[i] = mac_max(vol[i] * 1.0f, 0.0f);
}

// WarpAndProjct (WaP_Tomo.cpp:1207-1421) with imROI == 1.
void orc_warp_and_project(const orc_scan *s, const double *angles, const real *projs, int proj, real rtime,
                          const real *flow_fwd, const real *flow_adj, real *vol) {
  const int W = s->det[0], H = s->det[1];
  const size_t np = (size_t)W * H;
  const int *d = s->vol;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  const real aabb[6] = {0, (real)d[0], 0, (real)d[1], 0, (real)d[2]};
  std::vector<real> warped(nv), img(np), len(np), wt(np), c(np), delta(nv, 0.0f), back(nv);
  orc_advect(d, aabb, flow_fwd, vol, 1, rtime, warped.data(), s->threads);
  orc_forward(s, angles[proj], warped.data(), img.data(), len.data(), wt.data());
  orc_correction((int)np, projs + np * proj, img.data(), len.data(), nullptr, s->alpha, c.data());
  const int full[6] = {0, d[0], 0, d[1], 0, d[2]};
  orc_bp_voxel(s, angles[proj], c.data(), full, 1, delta.data());
  orc_advect(d, aabb, flow_adj, delta.data(), 1, -rtime, back.data(), s->threads);
  const double alpha = s->alpha;
  const real gmax = s->gmax;
  for (size_t i = 0; i < nv; ++i) {
    real x = (real)((double)vol[i] + (double)back[i] * alpha);
    x = (x < 0.0f) ? 0.0f : ((x > gmax) ? gmax : x);  // CImg::cut(0, G_Max)
    vol[i] = mac_max(x * 1.0f, 0.0f);
  }
}

// PSART::AdaptiveWarp (WaP_Tomo.cpp:878-1204, commented out in the
// reference), with the per-projection time the reference never fills
// (m_ProjIndex[i].rElapsed) taken as clamp((i - ftime) / tunit, -1, 1).
void orc_adaptive_warp(const orc_scan *s, const double *angles, const real *projs, int pstart, int pend, real ftime,
                       real tunit, int nb_warp, const int box[6], const real *flow_fwd, const real *flow_adj,
                       real *vol) {
  const int W = s->det[0], H = s->det[1];
  const size_t np = (size_t)W * H;
  const int *d = s->vol;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  const real aabb[6] = {0, (real)d[0], 0, (real)d[1], 0, (real)d[2]};
  std::vector<real> warped(nv), img(np), len(np), wt(np), c(np), delta(nv), back(nv), dual(np, 0.0f);
  const double alpha = s->alpha;
  const real gmax = s->gmax;
  for (int iter = 1; iter <= nb_warp; ++iter) {
    std::fill(delta.begin(), delta.end(), (real)0);  // deltaVol.fill(0.0f) (:911)
    for (int i = pstart; i <= pend; ++i) {
      real td = (i - ftime) / tunit;
      td = mac_min(mac_max(-1.0f, td), 1.0f);
      orc_advect(d, aabb, flow_fwd, vol, 1, td, warped.data(), s->threads);
      orc_forward(s, angles[i], warped.data(), img.data(), len.data(), wt.data());
      orc_correction((int)np, projs + np * i, img.data(), len.data(), dual.data(), s->alpha, c.data());
      orc_bp_voxel(s, angles[i], c.data(), box, 1, delta.data());
      orc_advect(d, aabb, flow_adj, delta.data(), 1, -td, back.data(), s->threads);
      for (size_t t = 0; t < nv; ++t) {
        const real x = (real)((double)vol[t] + (double)back[t] * alpha);
        vol[t] = (x < 0.0f) ? 0.0f : ((x > gmax) ? gmax : x);  // cut(0.0, G_Max) (:1161)
      }
    }
  }
  for (size_t t = 0; t < nv; ++t) vol[t] = mac_max(vol[t] * 1.0f, 0.0f);
}

// CP dual for frame f (WaP_Tomo.cpp:586-619).
void orc_cp_dual(const orc_scan *s, const int box[6], const real *xbar_f, const real *xbar_next, real *ytv_f,
                 real *ytp_f) {
  const int *d = s->vol;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  const real L = 8.0f, tau = 1.0f;
  const real sigma = .9 / (L * tau);
  const real tv_w = (real)s->tv_w, tp_w = (real)s->tp_w, huber = 1.0f;
  for (size_t i = 0; i < nv; ++i) ytp_f[i] += sigma * (xbar_next[i] - xbar_f[i]);
  const Grid g{{d[0], d[1], d[2]}};
  for (int k = box[4]; k < box[5]; ++k)
    for (int j = box[2]; j < box[3]; ++j)
      for (int i = box[0]; i < box[1]; ++i) {
        size_t t = g.id(i, j, k);
        ytv_f[t] += sigma * (xbar_f[g.id(i + 1, j, k)] - xbar_f[t]) * huber;
        ytv_f[nv + t] += sigma * (xbar_f[g.id(i, j + 1, k)] - xbar_f[t]) * huber;
        ytv_f[2 * nv + t] += sigma * (xbar_f[g.id(i, j, k + 1)] - xbar_f[t]) * huber;
        for (int c = 0; c < 3; ++c) ytv_f[c * nv + t] = mac_max(-tv_w, mac_min(tv_w, ytv_f[c * nv + t]));
        ytp_f[t] = ytp_f[t] * tp_w / (tp_w + 2 * sigma);
      }
}

// CP primal for frame f before its SART call (WaP_Tomo.cpp:622-660).
void orc_cp_primal(const orc_scan *s, const int box[6], int frame, const real *ytp_prev, const real *ytp_f,
                   const real *ytv_f, real *vol, real *xprev) {
  const int *d = s->vol;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  const real tau = 1.0f;
  std::memcpy(xprev, vol, nv * sizeof(real));
  if (frame == 0) {
    for (size_t i = 0; i < nv; ++i) vol[i] -= tau * (0.0f - ytp_f[i]);
  } else {
    for (size_t i = 0; i < nv; ++i) vol[i] -= tau * (ytp_prev[i] - ytp_f[i]);
  }
  const Grid g{{d[0], d[1], d[2]}};
  const real gmax = s->gmax;
  for (int k = box[4]; k < box[5]; ++k)
    for (int j = box[2]; j < box[3]; ++j)
      for (int i = box[0]; i < box[1]; ++i) {
        size_t t = g.id(i, j, k);
        real y1 = -(ytv_f[t] - ytv_f[g.id(i - 1, j, k)] + ytv_f[nv + t] - ytv_f[nv + g.id(i, j - 1, k)] +
                     ytv_f[2 * nv + t] - ytv_f[2 * nv + g.id(i, j, k - 1)]);
        vol[t] -= (tau * y1);
        vol[t] = mac_max(mac_min(gmax, vol[t]), 0);
      }
}

// X_bar = 2 x - x_prev over the ROI (WaP_Tomo.cpp:675-689).
void orc_cp_overrelax(const int dims[3], const int box[6], const real *vol, const real *xprev, real *xbar) {
  const Grid g{{dims[0], dims[1], dims[2]}};
  for (int k = box[4]; k < box[5]; ++k)
    for (int j = box[2]; j < box[3]; ++j)
      for (int i = box[0]; i < box[1]; ++i) {
        size_t t = g.id(i, j, k);
        xbar[t] = 2 * vol[t] - xprev[t];
      }
}

int orc_outer_iteration(const orc_scan *s, const orc_schedule *sch, const double *angles, const real *projs,
                        int level, real *vols, real *flows, real *ytv, real *ytp, real *xbar, real *xprev,
                        int *flow_iters_total) {
  return orc_outer_iteration_frames(s, sch, angles, projs, level, 0, 1 << 30, vols, flows, ytv, ytp, xbar, xprev,
                                    flow_iters_total);
}

// The outer iteration restricted to frames [f0, f1) (f1 clipped to F): their
// CP + SART steps, the flows of the pairs (f, f+1) they start, their
// warp-and-project windows; frames outside the range are read (CP neighbours,
// the pair's second frame) but not updated.  [0, F) is one outer iteration.
int orc_outer_iteration_frames(const orc_scan *s, const orc_schedule *sch, const double *angles, const real *projs,
                               int level, int f0, int f1, real *vols, real *flows, real *ytv, real *ytp, real *xbar,
                               real *xprev, int *flow_iters_total) {
  const int *d = s->vol;
  const size_t nv = (size_t)d[0] * d[1] * d[2];
  std::vector<int> st(130), en(130);
  std::vector<real> ft(130);
  real tunit;
  const int F = orc_level_frames(s->nframes_cli, s->nproj, level, st.data(), en.data(), ft.data(), &tunit);
  // m_roi = cut * dims / level-0 dims (WaP_Tomo.cpp:529-536), level-0 dims == dims.
  const int r = (int)((real)sch->cut * ((real)d[0] / (real)d[0]));
  const int box[6] = {r, d[0] - r, r, d[1] - r, r, d[2] - r};
  const size_t np = (size_t)s->det[0] * s->det[1];
  std::vector<real> dual((size_t)s->nproj * np);
  std::vector<real> zero(nv, 0.0f);
  f1 = std::min(f1, F);
  for (int icp = 1; icp <= sch->n_cp; ++icp)
    for (int f = f0; f < f1; ++f) {
      const real *xb_next = (f + 1 < F) ? xbar + (f + 1) * nv : zero.data();
      orc_cp_dual(s, box, xbar + f * nv, xb_next, ytv + f * 3 * nv, ytp + f * nv);
      orc_cp_primal(s, box, f, f > 0 ? ytp + (f - 1) * nv : nullptr, ytp + f * nv, ytv + f * 3 * nv, vols + f * nv,
                    xprev + f * nv);
      orc_sart_prox(s, angles, projs, st[f], en[f], sch->nb_sart, box, vols + f * nv, dual.data());
      orc_cp_overrelax(d, box, vols + f * nv, xprev + f * nv, xbar + f * nv);
    }
  int total = 0;
  const int cut6[6] = {sch->cut, sch->cut, sch->cut, sch->cut, sch->cut, sch->cut};
  for (int f = f0; f < f1 && f + 1 < F; ++f) {
    std::vector<real> out(3 * nv);
    total += orc_flow_multiscale(d, vols + f * nv, vols + (f + 1) * nv, flows + f * 3 * nv, sch->flow_tol,
                                 sch->flow_lambda, sch->flow_iters, sch->flow_warps, sch->flow_eta, sch->flow_sigma,
                                 sch->flow_scales, cut6, sch->deterministic, out.data());
    std::memcpy(flows + f * 3 * nv, out.data(), 3 * nv * sizeof(real));
  }
  for (int wp = 0; wp < sch->nb_projwarp; ++wp)
    for (int f = f0; f < sch->wp_frames && f < f1; ++f)
      for (int ik = st[f]; ik <= en[f]; ++ik) {
        real td = (ik - ft[f]) / tunit;
        td = mac_min(mac_max(-1.0f, td), 1.0f);
        const real *ffwd = flows + (size_t)(td < 0.0f ? std::max(0, f - 1) : f) * 3 * nv;
        const real *fadj = flows + (size_t)std::max(0, f - 1) * 3 * nv;
        orc_warp_and_project(s, angles, projs, ik, td, ffwd, fadj, vols + f * nv);
      }
  if (flow_iters_total) *flow_iters_total = total;
  return F;
}

// image_cg::cg<real> (cg.h:11-55) with image_blas dot/add (image_blas.h:9-91).
int orc_cg_screened_laplacian(const int dims[3], real a, real b, const real *rhs, real *x, real rel_tol,
                              int max_iters, real abs_tol, int mode) {
  const int W = dims[0], H = dims[1], D = dims[2];
  const size_t n = (size_t)W * H * D;
  auto id = [&](int i, int j, int k) { return i + (size_t)W * (j + (size_t)H * k); };
  auto apply = [&](const std::vector<real> &in, std::vector<real> &out) {
    for (int k = 0; k < D; ++k)
      for (int j = 0; j < H; ++j)
        for (int i = 0; i < W; ++i) {
          real xc = in[id(i, j, k)];
          real sn = in[id(i > 0 ? i - 1 : i, j, k)] + in[id(i < W - 1 ? i + 1 : i, j, k)] +
                     in[id(i, j > 0 ? j - 1 : j, k)] + in[id(i, j < H - 1 ? j + 1 : j, k)] +
                     in[id(i, j, k > 0 ? k - 1 : k)] + in[id(i, j, k < D - 1 ? k + 1 : k)];
          out[id(i, j, k)] = a * xc - b * (sn - 6.0f * xc);
        }
  };
  // image_blas::dot iterates x outermost, then y, then z.
  auto dot = [&](const std::vector<real> &u, const std::vector<real> &v) {
    real res = 0.0f;
    for (int i = 0; i < W; ++i)
      for (int j = 0; j < H; ++j)
        for (int k = 0; k < D; ++k) res += u[id(i, j, k)] * v[id(i, j, k)];
    return res;
  };
  std::vector<real> X(x, x + n), Ap(n), p(n), r(n);
  apply(X, Ap);
  for (size_t i = 0; i < n; ++i) r[i] = (real)((double)rhs[i] + (double)Ap[i] * -1.0);
  p = r;
  real rr, rr_old, rr_init, alpha;
  rr = rr_old = rr_init = dot(r, r);
  int iters = 0;
  if (std::sqrt(rr) < abs_tol) {
    std::memcpy(x, X.data(), n * sizeof(real));
    return 0;
  }
  for (int iter = 0; iter < max_iters; ++iter) {
    iters = iter + 1;
    apply(p, Ap);
    alpha = rr_old / dot(p, Ap);
    for (size_t i = 0; i < n; ++i) X[i] += p[i] * alpha;
    for (size_t i = 0; i < n; ++i) r[i] += Ap[i] * -alpha;
    rr = dot(r, r);
    if (std::sqrt(rr / rr_init) < rel_tol) break;
    const real beta = rr / rr_old;
    if (mode == 1)
      for (size_t i = 0; i < n; ++i) p[i] = r[i] + 0.0f * beta;
    else
      for (size_t i = 0; i < n; ++i) p[i] = r[i] + p[i] * beta;
    rr_old = rr;
  }
  std::memcpy(x, X.data(), n * sizeof(real));
  return iters;
}

}  // extern "C"
