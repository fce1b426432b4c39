// Host-side formats and tables of the command line (include/wap/wap_io.h).
//
// Analyze 7.5 / NIfTI-1 follows the byte layout CImg reads and writes
// (CImg.h:47829-47955 load, 51715-51790 save) so files interchange with the
// reference: header size at 0, dim[] (u16) at 40, datatype (u16) at 70,
// bitpix (u16) at 72, pixdim[] (f32) at 76, vox_offset (f32) at 108, scale
// (f32) at 112.  The angle reader and the z-split restate
// WaP_Tomo.cpp:324-339 and CImg.h:31389-31431; the angle generator restates
// Low_discrepency_squence.m:15-45.
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "wap/wap_io.h"
#include "c_boundary.h"

namespace {

std::string lower(std::string s) {
  for (char &ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

// Split at the last '.', like cimg::split_filename: body and extension.
void split_name(const std::string &path, std::string &body, std::string &ext) {
  const size_t dot = path.rfind('.');
  if (dot == std::string::npos) {
    body = path;
    ext.clear();
  } else {
    body = path.substr(0, dot);
    ext = path.substr(dot + 1);
  }
}

void swap_bytes(void *p, size_t elem, size_t n) {
  unsigned char *b = static_cast<unsigned char *>(p);
  for (size_t i = 0; i < n; ++i, b += elem)
    for (size_t k = 0; k < elem / 2; ++k) std::swap(b[k], b[elem - 1 - k]);
}

template <class T>
T field(const std::vector<unsigned char> &h, size_t off) {
  T v;
  std::memcpy(&v, h.data() + off, sizeof(T));
  return v;
}

struct Header {
  int dims[4] = {1, 1, 1, 1};
  int datatype = 0;
  float scale = 1.0f;
  bool swap = false;
  long data_offset = 0;  // into the data file
  std::string data_path;
};

int read_header(const char *path, Header &hd) {
  if (!path) return WAP_EINVAL;
  std::string body, ext, hpath = path;
  split_name(path, body, ext);
  const std::string e = lower(ext);
  bool single = false;
  if (e == "hdr") {
    hd.data_path = body + ".img";
  } else if (e == "img") {
    hpath = body + ".hdr";
    hd.data_path = path;
  } else {
    single = true;  // NIfTI single file
    hd.data_path = path;
  }
  std::FILE *f = std::fopen(hpath.c_str(), "rb");
  if (!f) return WAP_EIO;
  uint32_t hsize = 0;
  if (std::fread(&hsize, 4, 1, f) != 1 || hsize == 0) {
    std::fclose(f);
    return WAP_EIO;
  }
  if (hsize >= 4096) {
    hd.swap = true;
    swap_bytes(&hsize, 4, 1);
  }
  if (hsize < 116 || hsize > (1u << 20)) {
    std::fclose(f);
    return WAP_EIO;
  }
  std::vector<unsigned char> h(hsize, 0);
  const size_t got = std::fread(h.data() + 4, 1, hsize - 4, f);
  std::fclose(f);
  if (got != hsize - 4) return WAP_EIO;
  if (hd.swap) {
    swap_bytes(h.data() + 40, 2, 5);
    swap_bytes(h.data() + 70, 2, 1);
    swap_bytes(h.data() + 72, 2, 1);
    swap_bytes(h.data() + 76, 4, 4);
    swap_bytes(h.data() + 108, 4, 1);
    swap_bytes(h.data() + 112, 4, 1);
  }
  const unsigned short nd = field<unsigned short>(h, 40);
  for (int a = 0; a < 4 && a < nd; ++a) hd.dims[a] = field<unsigned short>(h, 42 + 2 * a);
  for (int a = 0; a < 4; ++a)
    if (hd.dims[a] <= 0) return WAP_EIO;
  hd.scale = field<float>(h, 112);
  if (hd.scale == 0.0f) hd.scale = 1.0f;
  hd.datatype = field<unsigned short>(h, 70);
  hd.data_offset = single ? (long)(unsigned)field<float>(h, 108) : 0;
  return WAP_OK;
}

template <class T, class Conv>
int read_data(std::FILE *f, float *out, size_t n, bool swap, Conv conv) {
  std::vector<T> buf(n);
  if (std::fread(buf.data(), sizeof(T), n, f) != n) return WAP_EIO;
  if (swap && sizeof(T) > 1) swap_bytes(buf.data(), sizeof(T), n);
  for (size_t i = 0; i < n; ++i) out[i] = conv(buf[i]);
  return WAP_OK;
}

}  // namespace

extern "C" {

int wap_analyze_info(const char *path, int *dims4, int *datatype) try {
  Header hd;
  const int r = read_header(path, hd);
  if (r != WAP_OK) return r;
  if (dims4)
    for (int a = 0; a < 4; ++a) dims4[a] = hd.dims[a];
  if (datatype) *datatype = hd.datatype;
  return WAP_OK;
} WAP_CATCH

int wap_analyze_load(const char *path, float *h_out, size_t count) try {
  if (!h_out) return WAP_EINVAL;
  Header hd;
  int r = read_header(path, hd);
  if (r != WAP_OK) return r;
  const size_t n = (size_t)hd.dims[0] * hd.dims[1] * hd.dims[2] * hd.dims[3];
  if (count < n) return WAP_EINVAL;
  std::FILE *f = std::fopen(hd.data_path.c_str(), "rb");
  if (!f) return WAP_EIO;
  if (hd.data_offset && std::fseek(f, hd.data_offset, SEEK_SET) != 0) {
    std::fclose(f);
    return WAP_EIO;
  }
  const float s = hd.scale;
  // (T)(buffer[off]*scalefactor) with T = float, as CImg converts each type.
  switch (hd.datatype) {
    case 2: r = read_data<unsigned char>(f, h_out, n, false, [s](unsigned char v) { return (float)(v * s); }); break;
    case 4: r = read_data<short>(f, h_out, n, hd.swap, [s](short v) { return (float)(v * s); }); break;
    case 8: r = read_data<int>(f, h_out, n, hd.swap, [s](int v) { return (float)(v * s); }); break;
    case 16: r = read_data<float>(f, h_out, n, hd.swap, [s](float v) { return v * s; }); break;
    case 64: r = read_data<double>(f, h_out, n, hd.swap, [s](double v) { return (float)(v * s); }); break;
    default: r = WAP_EIO;
  }
  std::fclose(f);
  return r;
} WAP_CATCH

int wap_analyze_save(const char *path, const float *h_data, const int *dims4, const float *voxel_size) try {
  if (!path || !h_data || !dims4) return WAP_EINVAL;
  for (int a = 0; a < 4; ++a)
    if (dims4[a] < 1 || dims4[a] > 32767) return WAP_EINVAL;
  std::string body, ext;
  split_name(path, body, ext);
  const std::string e = lower(ext);
  std::string hname, iname;
  if (e == "nii") {
    hname = path;
  } else if (e == "hdr" || e == "img") {
    hname = body + "." + (e == "hdr" ? ext : std::string("hdr"));
    iname = body + "." + (e == "img" ? ext : std::string("img"));
  } else {
    hname = std::string(path) + ".hdr";
    iname = std::string(path) + ".img";
  }
  const size_t hlen = iname.empty() ? 352 : 348;
  std::vector<unsigned char> h(hlen, 0);
  auto put16 = [&](size_t off, short v) { std::memcpy(h.data() + off, &v, 2); };
  auto putf = [&](size_t off, float v) { std::memcpy(h.data() + off, &v, 4); };
  const int32_t hs = 348;
  std::memcpy(h.data(), &hs, 4);
  std::memcpy(h.data() + 4, "CImg", 5);
  std::memcpy(h.data() + 14, " ", 2);
  put16(36, 4096);
  h[38] = 114;
  put16(40, 4);
  for (int a = 0; a < 4; ++a) put16(42 + 2 * a, (short)dims4[a]);
  put16(70, 16);                 // float
  put16(72, (short)sizeof(float));  // CImg stores sizeof(T) here
  putf(108, iname.empty() ? (float)hlen : 0.0f);
  putf(112, 1.0f);
  putf(76, 0.0f);
  for (int a = 0; a < 3; ++a) putf(80 + 4 * a, voxel_size ? voxel_size[a] : 1.0f);
  std::FILE *f = std::fopen(hname.c_str(), "wb");
  if (!f) return WAP_EIO;
  bool ok = std::fwrite(h.data(), 1, hlen, f) == hlen;
  if (!iname.empty()) {
    std::fclose(f);
    f = std::fopen(iname.c_str(), "wb");
    if (!f) return WAP_EIO;
  }
  const size_t n = (size_t)dims4[0] * dims4[1] * dims4[2] * dims4[3];
  ok = ok && std::fwrite(h_data, sizeof(float), n, f) == n;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? WAP_OK : WAP_EIO;
} WAP_CATCH

int wap_read_angles(const char *path, double *h_out, int n, int *h_read) try {
  if (!path || (!h_out && n > 0) || n < 0) return WAP_EINVAL;
  std::ifstream in(path);
  if (!in) return WAP_EIO;
  int i = 0;
  for (; i < n; ++i)
    if (!(in >> h_out[i])) break;
  for (int k = i; k < n; ++k) h_out[k] = 0.0;
  if (h_read) *h_read = i;
  return WAP_OK;
} WAP_CATCH

int wap_split_z(int depth, int nb, int *h_first, int *h_count) try {
  if (depth < 1 || nb < 1 || nb > depth || !h_first || !h_count) return WAP_EINVAL;
  if (nb == 1) {
    h_first[0] = 0;
    h_count[0] = depth;
    return WAP_OK;
  }
  int err = depth, start = 0, k = 0;
  for (int p = 0; p < depth; ++p) {
    err -= nb;
    if (err <= 0) {
      h_first[k] = start;
      h_count[k] = p - start + 1;
      ++k;
      err += depth;
      start = p + 1;
    }
  }
  return k == nb ? WAP_OK : WAP_EINVAL;
} WAP_CATCH

int wap_lds_angles(int np, int ns, int p, int nz, double *h_out) try {
  if (np < 0 || ns < 1 || p < 2 || nz < 1 || (!h_out && np > 0)) return WAP_EINVAL;
  int len = 0;
  long long i = 0;
  while (len < np) {
    if (len > 0 && len % nz == 0) h_out[len++] = 0.0;
    long long b = i++;
    double r = 0.0, q = 1.0 / p;
    while (b != 0) {
      r = r + (double)(b % p) * q;
      q = q / p;
      b = b / p;
    }
    r = 360.0 * r / ns;
    for (int k = 0; len < np && k < ns; ++k) h_out[len++] = r + k * 360.0 / ns;
  }
  return WAP_OK;
} WAP_CATCH

}  // extern "C"
