// Host-side block-sparse quantum-number tensors and the block-task planner.
//
// A tensor is the device counterpart of the reference's btas::QSTArray<double,N,fermion>
// (include/btas/QSPARSE/QSTArray.h:17-328): a total quantum number, per-index sector
// quantum numbers and dims, and the stored blocks keyed by their row-major sparse tag
// (include/btas/SPARSE/STArray.h:338-348).  The blocks live packed in ascending tag
// order in ONE device allocation, each block dense row-major; the host keeps tags,
// element offsets and dims so every plan below is pure host integer work.
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace mpsxx {

struct Qn {
  int p = 0;  // particle number
  int s = 0;  // 2*Sz
};
inline Qn operator+(Qn a, Qn b) { return {a.p + b.p, a.s + b.s}; }
inline Qn operator-(Qn a) { return {-a.p, -a.s}; }
inline bool operator==(Qn a, Qn b) { return a.p == b.p && a.s == b.s; }
inline bool operator!=(Qn a, Qn b) { return !(a == b); }
// order of src/fermion.h:97-101: by particle number, then spin
inline bool operator<(Qn a, Qn b) { return a.p == b.p ? a.s < b.s : a.p < b.p; }
inline bool parity(Qn a) { return (a.p & 1) != 0; }

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum Status {
  kOk = 0,
  kQShapeMismatch = 1,
  kAlloc = 2,
  kNoConvergence = 3,
  kDeviceTimeout = 4,
  kInvalidArgument = 5,
  kCuda = 6,
  kSolver = 7,
  kInternal = 8,
};

constexpr int kMaxRank = 6;

// Quantum + dense shape of a block-sparse tensor.
struct Shape {
  int rank = 0;
  Qn q;
  std::vector<std::vector<Qn>> qshape;
  std::vector<std::vector<int>> dshape;
  std::vector<int64_t> stride;
  int64_t nsparse = 0;

  void finalize();
  void index(int64_t tag, int* idx) const {
    for (int i = 0; i < rank; ++i) {
      idx[i] = static_cast<int>(tag / stride[i]);
      tag %= stride[i];
    }
  }
  int64_t tag(const int* idx) const {
    int64_t t = 0;
    for (int i = 0; i < rank; ++i) t += idx[i] * stride[i];
    return t;
  }
  bool allowed(const int* idx) const {
    Qn s;
    for (int i = 0; i < rank; ++i) s = s + qshape[i][idx[i]];
    return s == q;
  }
  bool allowed_tag(int64_t t) const {
    int idx[kMaxRank];
    index(t, idx);
    return allowed(idx);
  }
  int64_t block_size(const int* idx) const {
    int64_t n = 1;
    for (int i = 0; i < rank; ++i) n *= dshape[i][idx[i]];
    return n;
  }
  int nsec(int i) const { return static_cast<int>(qshape[i].size()); }
  Shape conjugate() const;
};

// Tensor descriptor: shape + stored blocks + (optional) device storage.
struct Tensor {
  Shape sh;
  std::vector<int64_t> tags;     // ascending
  std::vector<int64_t> offsets;  // element offset of each block
  std::unordered_map<int64_t, int32_t> slot;
  int64_t nnz = 0;
  double* d = nullptr;  // device data (nnz doubles), owned when own == true
  bool own = false;
  // Structural identity of the block layout (a hash of shape and stored tags):
  // tensors with equal layouts share it, so plans keyed by it are reused across
  // bonds and sweeps.
  uint64_t layout_id = 0;
  // Process-wide unique identity of the current data (new storage or an upload);
  // copies derived from the data (packed operands) are keyed by it.
  uint64_t data_version = 0;

  void set_blocks(const std::vector<int64_t>& sorted_tags);
  void allocate_allowed();  // every allowed block of non-zero size (STArray.h:219-237)
  int32_t find(int64_t t) const {
    auto it = slot.find(t);
    return it == slot.end() ? -1 : it->second;
  }
  void block_dims(int32_t b, int* dims) const {
    int idx[kMaxRank];
    sh.index(tags[b], idx);
    for (int i = 0; i < sh.rank; ++i) dims[i] = sh.dshape[i][idx[i]];
  }
  int64_t block_size(int32_t b) const {
    int idx[kMaxRank];
    sh.index(tags[b], idx);
    return sh.block_size(idx);
  }
};

uint64_t next_data_version();
uint64_t structure_hash(const Shape& sh, const std::vector<int64_t>& tags);

// ---------------------------------------------------------------------------
// Block-task enumeration of ST_Gemm_thread (include/btas/SPARSE/STBLAS.h:297-359)
// ---------------------------------------------------------------------------
enum Trans : int { kNoTrans = 0, kTrans = 1 };

struct GemmPairRef {
  int64_t a_tag, b_tag;  // tags of the original (un-viewed) operands
};
struct GemmTaskRef {
  int64_t c_tag;
  std::vector<GemmPairRef> pairs;
};

// Result shape of a Gemm (gemm_contract_qshape / gemm_contract_dshape).
Shape gemm_result_shape(Trans ta, Trans tb, const Shape& a, const Shape& b, int nc, int* K);

// Enumeration over the views QSTBLAS.h:215-225 passes for each transpose combination.
std::vector<GemmTaskRef> enumerate_gemm(Trans ta, Trans tb, const Tensor& a, const Tensor& b,
                                        const Shape& c, int K);

// ---------------------------------------------------------------------------
// Merge info (include/btas/QSPARSE/QSTmergeInfo.h:44-90)
// ---------------------------------------------------------------------------
struct MergeInfo {
  std::vector<std::vector<Qn>> qshape;
  std::vector<std::vector<int>> dshape;
  std::vector<Qn> q_packed;
  std::vector<int> d_packed;
  std::vector<Qn> q_merged;  // merged sectors in first-appearance order
  std::vector<int> d_merged;
  std::vector<int> merged_of;      // packed -> merged sector
  std::vector<int> offset_packed;  // packed -> offset inside its merged sector
  std::vector<std::vector<int>> members;
  MergeInfo() = default;
  MergeInfo(const std::vector<std::vector<Qn>>& qs, const std::vector<std::vector<int>>& ds);
};

}  // namespace mpsxx
