// Host geometry of the cone-beam scan (geometry.cpp).
#pragma once

#include "wap_internal.h"

namespace wap {

struct ScanGeometry {
  int vol[3];
  int det[2];
  double vs, ds, sid, sdd;
  double oxyz[3];
};

ProjGeom projection_geometry(const ScanGeometry &sg, double angle_deg);
double half_frustum(int pixels, double ds);
float sample_distance(double vs);
int level_frames(int nframes_cli, int nproj, int level, int *start, int *end, float *ftime, float *tunit, int cap);

}  // namespace wap
