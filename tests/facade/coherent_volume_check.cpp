// Reads bs[3], dims[3] (int32) and dims[0]*dims[1]*dims[2] floats from argv[1];
// writes every GetValue (float), the block range (two doubles) and the count
// of blocks that keep data (int32) to argv[2].
#include <cstdio>
#include <vector>

#include "wap/coherent_volume.hpp"

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int bs[3], dims[3];
  if (std::fread(bs, 4, 3, f) != 3 || std::fread(dims, 4, 3, f) != 3) return 4;
  const size_t n = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<float> data(n), out(n);
  if (std::fread(data.data(), 4, n, f) != n) return 5;
  std::fclose(f);
  wap19::CoherentVolume cv(bs[0], bs[1], bs[2]);
  cv.SetDimensions(dims);
  cv.AllocateBlocks();
  cv.SetData(data.data());
  for (int z = 0; z < dims[2]; ++z)
    for (int y = 0; y < dims[1]; ++y)
      for (int x = 0; x < dims[0]; ++x) out[x + (size_t)dims[0] * (y + (size_t)dims[1] * z)] = cv.GetValue(x, y, z);
  double mm[2];
  cv.GetMinMaxValue(mm[0], mm[1]);
  const int stored = (int)cv.StoredBlocks();
  std::vector<float> dense(n);
  cv.CopyTo(dense.data());
  for (size_t i = 0; i < n; ++i)
    if (dense[i] != out[i]) return 6;
  FILE *g = std::fopen(argv[2], "wb");
  if (!g) return 7;
  std::fwrite(out.data(), 4, n, g);
  std::fwrite(mm, 8, 2, g);
  std::fwrite(&stored, 4, 1, g);
  std::fclose(g);
  return 0;
}
