// wap_tomo -- headless command line of the warp-and-project reconstruction,
// with the reference program's options (main.cpp:15-185) and its flow
// (main.cpp:186-220): VolumeData -> PSART -> SetData -> Render.  The GLUT
// window of the reference is replaced by running Render directly.
//
// Option parsing follows argtable2's getopt_long rules: "-f 64", "-f64",
// "--XYZ=64" and "--XYZ 64" are the same; multi-value options repeat
// ("-f 64 -f 64 -f 48"), and values not given keep the reference's defaults
// (main.cpp:107-150).  Options beyond the reference's (marked [ext]) cover
// what it hard-codes: the projection count (main.cpp:198: 192), the angle
// file name (WaP_Tomo.cpp:324: ours_foam_compress.txt), the dumps.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define WAP19_GLOBAL_NAMES
#include "wap/wap19.hpp"

namespace {

struct Opt {
  char s;             // short name (0: none)
  const char *l;      // long name
  int kind;           // 0 flag, 1 int, 2 double, 3 string
  int maxcount;
  const char *help;
};

const Opt kOpts[] = {
    {'s', "Sigma", 2, 1, "TV weight (default 0.3)"},
    {'t', "Tau", 2, 1, "temporal weight (default 0.3)"},
    {'l', "Lambda", 2, 1, "data/prior trade-off (unused, as in the reference; default 0.1)"},
    {'a', "Alpha", 2, 1, "SART relaxation (default 0.1)"},
    {'o', nullptr, 3, 1, "output file prefix (default Test/test)"},
    {'v', "nframes", 1, 1, "number of frames (default 1)"},
    {'r', "nrounds", 1, 1, "rounds per frame (default 1)"},
    {'f', "XYZ", 1, 3, "volume size, up to 3 values (default 63 63 63)"},
    {'u', "imgUV", 1, 2, "projection width and height"},
    {'c', "voxelspacing", 2, 1, "voxel spacing (default 1)"},
    {'d', "detector spacing", 2, 1, "detector spacing (default 1)"},
    {'i', "projsvolume", 3, 20, "projection stack (.hdr/.img Analyze, .nii or .tif/.tiff)"},
    {'j', "sdd", 2, 1, "source to detector distance (default 200)"},
    {'g', "sid", 2, 1, "source to iso-centre distance (default 400)"},
    {0, "oxyz", 2, 3, "volume centre offset x y z (default 0)"},
    {0, "sdg", 2, 20, "start degree of each projection sequence (unused by the live path)"},
    {'b', "AlgorithmIter", 1, 1, "algorithm iterations (unused by the live path; default 2)"},
    {'p', "SartIter", 1, 1, "SART nested iterations (default 2)"},
    {0, "prior", 3, 1, "{STV,SAD,ATV} (default ATV)"},
    {0, "bp", 3, 1, "{Voxelbased,Raybased} (default Voxelbased; Raybased: SART backprojects ray-driven)"},
    {'h', "help", 0, 1, "print this help and exit"},
    {0, "version", 0, 1, "print version information and exit"},
    {0, "nproj", 1, 1, "[ext] projections in the stack (default 192, the reference's constant)"},
    {0, "angles", 3, 1, "[ext] angle file (default ours_foam_compress.txt)"},
    {0, "levels", 1, 1, "[ext] time levels (default 2)"},
    {0, "dump", 3, 1, "[ext] {all,none}: the reference's Analyze dumps (default all)"},
    {0, "bp-arith", 3, 1, "[ext] {exact,fp32}: backprojection arithmetic (default exact, the reference's)"},
    {0, "flow-iters", 1, 1, "[ext] primal-dual iterations per flow level (default 3000)"},
    {0, "flow-scales", 1, 1, "[ext] flow pyramid levels (default 5)"},
    {0, "save-final", 3, 1, "[ext] write PREFIX.level%02d.f%03d.{vol,flow}.hdr after the last level"},
    {0, "flow-bits", 1, 1, "[ext] {32,16}: 16 = the precision form (FP16 flow-solver state; default 32)"},
};

struct Values {
  std::vector<std::vector<std::string>> v;
  Values() : v(sizeof(kOpts) / sizeof(kOpts[0])) {}
};

void usage(FILE *out) {
  std::fprintf(out, "Usage: wap_tomo [options]\n");
  for (const Opt &o : kOpts) {
    std::string n;
    if (o.s) n += std::string("-") + o.s;
    if (o.l) n += (n.empty() ? "" : ", ") + std::string("--") + o.l;
    if (o.kind) n += o.kind == 1 ? " <int>" : o.kind == 2 ? " <double>" : " <str>";
    std::fprintf(out, "  %-34s %s\n", n.c_str(), o.help);
  }
}

int find_short(char c) {
  for (size_t i = 0; i < sizeof(kOpts) / sizeof(kOpts[0]); ++i)
    if (kOpts[i].s == c) return (int)i;
  return -1;
}

int find_long(const std::string &name) {
  for (size_t i = 0; i < sizeof(kOpts) / sizeof(kOpts[0]); ++i)
    if (kOpts[i].l && name == kOpts[i].l) return (int)i;
  return -1;
}

bool parse(int argc, char **argv, Values &vals, std::string &err) {
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    int idx = -1;
    std::string val;
    bool has_val = false;
    if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
      std::string name = a.substr(2);
      const size_t eq = name.find('=');
      if (eq != std::string::npos) {
        val = name.substr(eq + 1);
        name = name.substr(0, eq);
        has_val = true;
      }
      idx = find_long(name);
      if (idx < 0) {
        err = "unknown option --" + name;
        return false;
      }
    } else if (a.size() >= 2 && a[0] == '-') {
      idx = find_short(a[1]);
      if (idx < 0) {
        err = std::string("unknown option -") + a[1];
        return false;
      }
      if (a.size() > 2) {
        val = a.substr(2);
        has_val = true;
      }
    } else {
      err = "unexpected argument " + a;
      return false;
    }
    const Opt &o = kOpts[idx];
    if (o.kind == 0) {
      vals.v[idx].push_back("1");
      continue;
    }
    if (!has_val) {
      if (i + 1 >= argc) {
        err = std::string("option ") + a + " needs a value";
        return false;
      }
      val = argv[++i];
    }
    if ((int)vals.v[idx].size() >= o.maxcount) {
      err = std::string("too many occurrences of ") + a;
      return false;
    }
    char *end = nullptr;
    errno = 0;
    if (o.kind == 1) std::strtol(val.c_str(), &end, 0);
    if (o.kind == 2) std::strtod(val.c_str(), &end);
    if (o.kind != 3 && (end == val.c_str() || *end != '\0' || errno)) {
      err = std::string("invalid value '") + val + "' for " + a;
      return false;
    }
    vals.v[idx].push_back(val);
  }
  return true;
}

const std::vector<std::string> &get(const Values &v, const char *lname, char s = 0) {
  const int i = lname ? find_long(lname) : find_short(s);
  return v.v[i];
}

double dbl(const Values &v, const char *l, char s, double def, int k = 0) {
  const auto &x = get(v, l, s);
  return (int)x.size() > k ? std::strtod(x[k].c_str(), nullptr) : def;
}

int integer(const Values &v, const char *l, char s, int def, int k = 0) {
  const auto &x = get(v, l, s);
  return (int)x.size() > k ? (int)std::strtol(x[k].c_str(), nullptr, 0) : def;
}

std::string str(const Values &v, const char *l, char s, const std::string &def) {
  const auto &x = get(v, l, s);
  return x.empty() ? def : x[0];
}

}  // namespace

int main(int argc, char **argv) {
  Values vals;
  std::string err;
  if (!parse(argc, argv, vals, err)) {
    std::fprintf(stdout, "wap_tomo: %s\nTry 'wap_tomo --help' for more information.\n", err.c_str());
    return 1;
  }
  if (!get(vals, "help").empty()) {
    usage(stdout);
    return 0;
  }
  if (!get(vals, "version").empty()) {
    std::printf("wap_tomo: GB300 warp-and-project reconstruction (C ABI %s)\n", "wap.h");
    return 0;
  }
  if (argc == 1) {
    std::printf("Try 'wap_tomo --help' for more information.\n");
    return 0;
  }
  // defaults of main.cpp:107-150, then the parsed values
  int vols[3] = {63, 63, 63};
  for (int k = 0; k < 3; ++k) vols[k] = integer(vals, "XYZ", 'f', vols[k], k);
  int imgWH[2];
  imgWH[0] = integer(vals, "imgUV", 'u', 512, 0);
  imgWH[1] = integer(vals, "imgUV", 'u', imgWH[0], 1);
  double oxyz[3];
  for (int k = 0; k < 3; ++k) oxyz[k] = dbl(vals, "oxyz", 0, 0.0, k);
  std::vector<double> sdg(20, 0.0);
  for (int k = 0; k < 20; ++k) sdg[k] = dbl(vals, "sdg", 0, 0.0, k);
  const double d1 = dbl(vals, "Sigma", 's', 0.3), d2 = dbl(vals, "Tau", 't', 0.3), d3 = dbl(vals, "Lambda", 'l', 0.1);
  const double alp = dbl(vals, "Alpha", 'a', 0.1), vs = dbl(vals, "voxelspacing", 'c', 1.0);
  const double ds = dbl(vals, "detector spacing", 'd', 1.0);
  const double sdd = dbl(vals, "sdd", 'j', 200.0), sid = dbl(vals, "sid", 'g', 400.0);
  const int nframe = integer(vals, "nframes", 'v', 1), nrounds = integer(vals, nullptr, 'r', 1);
  const int algo = integer(vals, "AlgorithmIter", 'b', 2), sartit = integer(vals, "SartIter", 'p', 2);
  const std::string outfile = str(vals, nullptr, 'o', "Test/test");
  const std::string prior = str(vals, "prior", 0, "ATV"), bp = str(vals, "bp", 0, "Voxelbased");
  const int totalproj = integer(vals, "nproj", 0, 192);
  const std::string angle_file = str(vals, "angles", 0, "ours_foam_compress.txt");
  const std::string dump = str(vals, "dump", 0, "all"), arith = str(vals, "bp-arith", 0, "exact");
  const auto &projfiles = get(vals, "projsvolume", 'i');
  if (projfiles.empty()) {
    std::printf("wap_tomo: missing option -i <projection stack>\n");
    return 1;
  }
  if (bp != "Voxelbased" && bp != "Raybased") {
    std::printf("wap_tomo: --bp must be Voxelbased or Raybased\n");
    return 1;
  }
  if ((dump != "all" && dump != "none") || (arith != "exact" && arith != "fp32")) {
    std::printf("wap_tomo: bad --dump or --bp-arith value\n");
    return 1;
  }
  std::vector<const char *> pfiles;
  for (const auto &p : projfiles) pfiles.push_back(p.c_str());
  pfiles.push_back(nullptr);
  try {
    // main.cpp:192-219
    VolumeData data;
    data.setParas(vols, vs, nframe, totalproj);
    const int nlevels = integer(vals, "levels", 0, 2);
    data.ReadStructuredFile(nlevels);
    PSART scene(d1, d2, d3, outfile.c_str(), imgWH, totalproj, algo, sartit, alp, sid, pfiles.data(), oxyz, sdd, ds,
                prior.c_str(), bp.c_str(), vols, nframe, sdg.data(), nrounds, angle_file.c_str());
    scene.m_nlevels = nlevels;
    scene.m_dump = dump == "all";
    scene.m_bp_exact = arith == "exact" ? 1 : 0;
    scene.m_flow_iters = integer(vals, "flow-iters", 0, 3000);
    scene.m_flow_scales = integer(vals, "flow-scales", 0, 5);
    scene.m_flow_bits = integer(vals, "flow-bits", 0, 32);
    if (scene.m_flow_bits != 32 && scene.m_flow_bits != 16) {
      std::printf("wap_tomo: --flow-bits must be 32 or 16\n");
      return 1;
    }
    // Render's local nb_proxiSART is 2 whatever -p says (WaP_Tomo.cpp:484)
    scene.SetData(&data);
    scene.Render();
    const std::string fin = str(vals, "save-final", 0, "");
    if (!fin.empty()) {
      const int L = std::min(nlevels, (int)data.m_Frameslist.size()) - 1;
      char name[1024];
      for (int f = 0; f < (int)data.m_Frameslist[L].size(); ++f) {
        std::snprintf(name, sizeof(name), "%s.level%02d.f%03d.vol.hdr", fin.c_str(), L, f);
        data.m_Frameslist[L][f].fVolume.save_analyze(name);
        std::snprintf(name, sizeof(name), "%s.level%02d.f%03d.flow.hdr", fin.c_str(), L, f);
        data.m_Frameslist[L][f].fFlow.save_analyze(name);
      }
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "wap_tomo: %s\n", e.what());
    return 2;
  }
  return 0;
}
