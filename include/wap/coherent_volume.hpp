// coherent_volume.hpp -- CoherentVolume, the reference's block-partitioned
// volume (CoherentVolume.h:16-85, CoherentVolume.cpp:33-258), header-only.
//
// The volume is cut into blocks of a fixed size (the last block along an
// axis holds the remainder); each block records the minimum and maximum of
// its values and drops its data when they are equal (a constant block).
// GetValue(x, y, z) reads through the block, GetMinMaxValue reduces the
// blocks' ranges.  Method names and argument meanings are the reference's
// (GetBlcokSize keeps its spelling; GetBlockSize is the same call).  It lives in
// namespace wap19 with the rest of the facade (wap19.hpp, which includes this
// header, also exports it globally under WAP19_GLOBAL_NAMES).
//
// Where the reference is defined this class gives its results: SetData and
// SetBlockSlice advance their source pointers by element counts multiplied by
// sizeof(float) (CoherentVolume.cpp:190,193,226), which stays inside the data
// only when every axis has one block.  For more blocks this class advances by
// element counts, the layout the loops are written for (rows of dims[0]
// floats, slices of dims[0] * dims[1]).  GetMinMaxValue on a volume whose
// blocks were never allocated returns 0, 0 (the reference dereferences a null
// block array).
#ifndef WAP_COHERENT_VOLUME_HPP
#define WAP_COHERENT_VOLUME_HPP

#include <algorithm>
#include <cstring>
#include <vector>

namespace wap19 {

class CoherentVolume {
 public:
  explicit CoherentVolume(int x, int y, int z) {
    m_BlockSize[0] = x;
    m_BlockSize[1] = y;
    m_BlockSize[2] = z;
  }
  virtual ~CoherentVolume() = default;

  virtual void Initialize() { m_Blocks.clear(); }

  void SetBlockSize(const int bs[3]) {
    for (int a = 0; a < 3; ++a) m_BlockSize[a] = bs[a];
  }
  void GetBlcokSize(int bs[3]) const {
    for (int a = 0; a < 3; ++a) bs[a] = m_BlockSize[a];
  }
  void GetBlockSize(int bs[3]) const { GetBlcokSize(bs); }
  void SetDimensions(const int dims[3]) {
    for (int a = 0; a < 3; ++a) {
      m_Dimensions[a] = dims[a];
      m_BlockNum[a] = (m_Dimensions[a] - 1) / m_BlockSize[a] + 1;
    }
  }
  void GetDimensions(int dims[3]) const {
    for (int a = 0; a < 3; ++a) dims[a] = m_Dimensions[a];
  }
  void SetSpacings(const float s[3]) {
    for (int a = 0; a < 3; ++a) m_Spacings[a] = s[a];
  }
  void GetSpacings(float s[3]) const {
    for (int a = 0; a < 3; ++a) s[a] = m_Spacings[a];
  }
  void GetBlockNum(int bn[3]) const {
    for (int a = 0; a < 3; ++a) bn[a] = m_BlockNum[a];
  }

  void AllocateBlocks() {
    Initialize();
    m_Blocks.assign((size_t)m_BlockNum[0] * m_BlockNum[1] * m_BlockNum[2], Block());
  }

  // Blocks of block-slice sliceID (the sliceID-th layer of blocks along z)
  // from sliceData, the first of its dimz voxel slices (dimz < 0: the block
  // size).
  void SetBlockSlice(void *sliceData, int sliceID, int dimz = -1) {
    if (m_Blocks.empty()) return;
    if (dimz < 0) dimz = m_BlockSize[2];
    const float *row = static_cast<const float *>(sliceData);
    for (int i = 0; i < m_BlockNum[1]; ++i, row += (size_t)m_BlockSize[1] * m_Dimensions[0]) {
      const float *p = row;
      for (int j = 0; j < m_BlockNum[0]; ++j, p += m_BlockSize[0])
        m_Blocks[((size_t)sliceID * m_BlockNum[1] + i) * m_BlockNum[0] + j].Set(
            p, std::min(m_BlockSize[0], m_Dimensions[0] - m_BlockSize[0] * j),
            std::min(m_BlockSize[1], m_Dimensions[1] - m_BlockSize[1] * i), std::min(m_BlockSize[2], dimz),
            m_Dimensions[0], m_Dimensions[0] * m_Dimensions[1]);
    }
  }

  // The whole volume (x fastest, dims[0] * dims[1] * dims[2] floats).
  void SetData(float *data) {
    if (m_Blocks.empty()) return;
    const float *p = data;
    for (int i = 0; i < m_BlockNum[2]; ++i, p += (size_t)m_BlockSize[2] * m_Dimensions[0] * m_Dimensions[1])
      SetBlockSlice(const_cast<float *>(p), i, std::min(m_BlockSize[2], m_Dimensions[2] - m_BlockSize[2] * i));
  }

  float GetValue(int x, int y, int z) const {
    if (m_Blocks.empty()) return 0.0f;
    const int bx = x / m_BlockSize[0], by = y / m_BlockSize[1], bz = z / m_BlockSize[2];
    return m_Blocks[bx + ((size_t)by + (size_t)bz * m_BlockNum[1]) * m_BlockNum[0]].Get(
        x % m_BlockSize[0], y % m_BlockSize[1], z % m_BlockSize[2]);
  }

  void GetMinMaxValue(double &minValue, double &maxValue) const {
    if (m_Blocks.empty()) {
      minValue = maxValue = 0.0;
      return;
    }
    float mn = m_Blocks[0].mn, mx = m_Blocks[0].mx;
    for (const Block &b : m_Blocks) {
      mn = mn < b.mn ? mn : b.mn;  // the reference's min/max macros
      mx = mx > b.mx ? mx : b.mx;
    }
    minValue = mn;
    maxValue = mx;
  }

  // Blocks that hold data (the others are constant): the compression the
  // class exists for.
  size_t StoredBlocks() const {
    size_t n = 0;
    for (const Block &b : m_Blocks) n += b.data.empty() ? 0 : 1;
    return n;
  }

  // The dense volume back (x fastest), for the library's device calls.
  void CopyTo(float *out) const {
    for (int z = 0; z < m_Dimensions[2]; ++z)
      for (int y = 0; y < m_Dimensions[1]; ++y)
        for (int x = 0; x < m_Dimensions[0]; ++x)
          out[x + (size_t)m_Dimensions[0] * (y + (size_t)m_Dimensions[1] * z)] = GetValue(x, y, z);
  }

 private:
  struct Block {
    std::vector<float> data;  // empty: constant block of value mn
    int yinc = 0, zinc = 0;
    float mn = 0.0f, mx = 0.0f;
    // CoherentVolume.cpp TBlock::SetData: copy rows, track the range from the
    // first value, drop the data of a constant block
    void Set(const float *src, int xs, int ys, int zs, int ysrc, int zsrc) {
      data.assign((size_t)xs * ys * zs, 0.0f);
      yinc = xs;
      zinc = xs * ys;
      mn = mx = src[0];
      for (int k = 0; k < zs; ++k)
        for (int j = 0; j < ys; ++j) {
          const float *s = src + (size_t)k * zsrc + (size_t)j * ysrc;
          float *d = data.data() + (size_t)k * zinc + (size_t)j * yinc;
          std::memcpy(d, s, sizeof(float) * xs);
          for (int i = 0; i < xs; ++i) {
            mn = mn < d[i] ? mn : d[i];
            mx = mx > d[i] ? mx : d[i];
          }
        }
      if (mn == mx) data.clear();
    }
    float Get(int x, int y, int z) const {
      return data.empty() ? mn : data[(size_t)z * zinc + (size_t)y * yinc + x];
    }
  };
  std::vector<Block> m_Blocks;
  int m_BlockSize[3] = {1, 1, 1};
  int m_Dimensions[3] = {0, 0, 0};
  float m_Spacings[3] = {1.0f, 1.0f, 1.0f};
  int m_BlockNum[3] = {0, 0, 0};
};

}  // namespace wap19

#endif  // WAP_COHERENT_VOLUME_HPP
