// ORACLE — test infrastructure only.  A lazily materialised implementation of the reference's traceback matrix
// class (model/Matrix.h of the dCNS sources, whose interface is kept unchanged), linked in place of its dense
// model/Matrix.cpp so that the unmodified alignment code can run on pairs whose dense (L1+1) x (L2+1) byte matrix
// would not fit in memory (200 kb pairs: 40 GB per matrix).
//
// Semantics kept exactly (model/Matrix.cpp:7-36): every cell starts at 0; reset(a, b) sets the cells of rows < a and
// columns < b to 255; set writes one cell; get returns a reference to one cell.  Only the cells an alignment touches
// are stored, in chunks of kChunk columns of one row.  Resets are recorded in order; a chunk remembers how many of
// them it has seen and applies the newer ones (in order) the next time it is accessed, so a cell's value is the same
// as the dense matrix's after any interleaving of resets and writes.  A chunk created after some resets starts from
// zeros overwritten by the union of all earlier reset rectangles (kept as a staircase of their corners).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <utility>
#include <vector>

#include "model/Matrix.h"

namespace {

constexpr int32_t kChunk = 256;

struct Chunk {
  size_t seen;  // resets applied so far
  uint8_t v[kChunk];
};

struct Lazy {
  std::unordered_map<uint64_t, Chunk *> chunks;
  std::vector<std::pair<int32_t, int32_t>> resets;  // (a, b) in call order
  // union of the reset rectangles [0, a) x [0, b): corners with a increasing and b decreasing
  std::vector<std::pair<int32_t, int32_t>> stair;

  ~Lazy() {
    for (auto &kv : chunks) delete kv.second;
  }

  // columns [0, B) of row i lie inside some earlier reset rectangle
  int32_t covered_cols(int32_t i) const {
    auto it = std::upper_bound(stair.begin(), stair.end(), std::make_pair(i, INT32_MAX));
    return it == stair.end() ? 0 : it->second;
  }

  void add_reset(int32_t a, int32_t b) {
    resets.emplace_back(a, b);
    for (auto &c : stair)
      if (c.first >= a && c.second >= b) return;  // already inside the union
    std::vector<std::pair<int32_t, int32_t>> next;
    for (auto &c : stair)
      if (!(c.first <= a && c.second <= b)) next.push_back(c);
    next.emplace_back(a, b);
    std::sort(next.begin(), next.end());
    stair.swap(next);
  }

  static void fill(Chunk *c, int32_t col0, int32_t upto) {
    const int32_t n = std::min(upto - col0, kChunk);
    if (n > 0) std::memset(c->v, 255, (size_t)n);
  }

  uint8_t &cell(int32_t i, int32_t j) {
    const int32_t cj = j / kChunk, col0 = cj * kChunk;
    const uint64_t key = ((uint64_t)(uint32_t)i << 32) | (uint32_t)cj;
    auto it = chunks.find(key);
    Chunk *c;
    if (it == chunks.end()) {
      c = new Chunk;
      std::memset(c->v, 0, sizeof(c->v));
      fill(c, col0, covered_cols(i));
      c->seen = resets.size();
      chunks.emplace(key, c);
    } else {
      c = it->second;
      for (; c->seen < resets.size(); ++c->seen) {
        const auto &r = resets[c->seen];
        if (i < r.first) fill(c, col0, r.second);
      }
    }
    return c->v[j - col0];
  }
};

inline Lazy *state(uint8_t **T) { return reinterpret_cast<Lazy *>(T); }

}  // namespace

Matrix::Matrix(int32_t _length1, int32_t _length2) {
  length1 = _length1;
  length2 = _length2;
  T = reinterpret_cast<uint8_t **>(new Lazy);
}

Matrix::~Matrix() { delete state(T); }

void Matrix::reset(int32_t a, int32_t b) {
  a = std::min(a, length1);
  b = std::min(b, length2);
  if (a > 0 && b > 0) state(T)->add_reset(a, b);
}

void Matrix::set(int32_t &a, int32_t &b, uint8_t &c) { state(T)->cell(a, b) = c; }

uint8_t &Matrix::get(int32_t &a, int32_t &b) { return state(T)->cell(a, b); }
