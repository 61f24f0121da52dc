// Host-side shapes, layouts and the ST_Gemm_thread block-task enumeration.
#include "qsd.hpp"

#include <algorithm>
#include <atomic>
#include <map>

namespace mpsxx {

uint64_t next_data_version() {
  static std::atomic<uint64_t> counter{1};
  return counter.fetch_add(1);
}

namespace {
uint64_t mix(uint64_t h, uint64_t v) {
  // splitmix64 finaliser over the running state
  uint64_t z = h ^ (v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2));
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
}  // namespace

uint64_t structure_hash(const Shape& sh, const std::vector<int64_t>& tags) {
  uint64_t h = mix(0x6d707378ull, static_cast<uint64_t>(sh.rank));
  h = mix(h, static_cast<uint32_t>(sh.q.p));
  h = mix(h, static_cast<uint32_t>(sh.q.s));
  for (int i = 0; i < sh.rank; ++i) {
    h = mix(h, sh.qshape[i].size());
    for (size_t j = 0; j < sh.qshape[i].size(); ++j) {
      h = mix(h, static_cast<uint32_t>(sh.qshape[i][j].p));
      h = mix(h, static_cast<uint32_t>(sh.qshape[i][j].s));
      h = mix(h, static_cast<uint32_t>(sh.dshape[i][j]));
    }
  }
  h = mix(h, tags.size());
  for (int64_t t : tags) h = mix(h, static_cast<uint64_t>(t));
  return h ? h : 1;
}

void Shape::finalize() {
  if (static_cast<int>(qshape.size()) != rank || static_cast<int>(dshape.size()) != rank)
    throw Error(kInvalidArgument, "shape: rank does not match qshape/dshape");
  if (rank > kMaxRank) throw Error(kInvalidArgument, "shape: rank exceeds the supported maximum");
  stride.assign(rank, 0);
  int64_t s = 1;
  for (int i = rank - 1; i >= 0; --i) {
    if (qshape[i].size() != dshape[i].size())
      throw Error(kInvalidArgument, "shape: qshape and dshape have different block size");
    stride[i] = s;
    s *= static_cast<int64_t>(qshape[i].size());
  }
  nsparse = rank ? s : 0;
}

Shape Shape::conjugate() const {
  Shape c = *this;
  c.q = -q;
  for (auto& v : c.qshape)
    for (auto& x : v) x = -x;
  return c;
}

void Tensor::set_blocks(const std::vector<int64_t>& sorted_tags) {
  tags = sorted_tags;
  offsets.resize(tags.size());
  slot.clear();
  slot.reserve(tags.size() * 2 + 1);
  int64_t off = 0;
  for (size_t b = 0; b < tags.size(); ++b) {
    if (b && tags[b] <= tags[b - 1]) throw Error(kInvalidArgument, "tensor: block tags must be strictly ascending");
    if (tags[b] < 0 || tags[b] >= sh.nsparse) throw Error(kInvalidArgument, "tensor: block tag out of range");
    int idx[kMaxRank];
    sh.index(tags[b], idx);
    if (!sh.allowed(idx)) throw Error(kQShapeMismatch, "tensor: block not allowed by its quantum numbers");
    offsets[b] = off;
    slot[tags[b]] = static_cast<int32_t>(b);
    off += sh.block_size(idx);
  }
  nnz = off;
  layout_id = structure_hash(sh, tags);
}

void Tensor::allocate_allowed() {
  std::vector<int64_t> t;
  int idx[kMaxRank] = {0};
  for (int64_t tag = 0; tag < sh.nsparse; ++tag) {
    sh.index(tag, idx);
    if (sh.allowed(idx) && sh.block_size(idx) > 0) t.push_back(tag);
  }
  set_blocks(t);
}

Shape gemm_result_shape(Trans ta, Trans tb, const Shape& a, const Shape& b, int nc, int* Kout) {
  // include/btas/QSPARSE/btas_contract_qshape.h:60-108 with real data (Trans == no sign flip)
  const int NA = a.rank, NB = b.rank;
  const int K = (NA + NB - nc) / 2;
  if (K <= 0 || K > NA || K > NB || NA + NB - 2 * K != nc)
    throw Error(kInvalidArgument, "gemm: inconsistent ranks");
  Shape c;
  c.rank = nc;
  std::vector<std::vector<Qn>> kq;
  if (ta == kNoTrans) {
    for (int i = 0; i < NA - K; ++i) { c.qshape.push_back(a.qshape[i]); c.dshape.push_back(a.dshape[i]); }
    for (int i = 0; i < K; ++i) kq.push_back(a.qshape[i + NA - K]);
  } else {
    for (int i = 0; i < NA - K; ++i) { c.qshape.push_back(a.qshape[i + K]); c.dshape.push_back(a.dshape[i + K]); }
    for (int i = 0; i < K; ++i) kq.push_back(a.qshape[i]);
  }
  std::vector<std::vector<Qn>> bk;
  if (tb == kNoTrans) {
    for (int i = 0; i < NB - K; ++i) { c.qshape.push_back(b.qshape[i + K]); c.dshape.push_back(b.dshape[i + K]); }
    for (int i = 0; i < K; ++i) bk.push_back(b.qshape[i]);
  } else {
    for (int i = 0; i < NB - K; ++i) { c.qshape.push_back(b.qshape[i]); c.dshape.push_back(b.dshape[i]); }
    for (int i = 0; i < K; ++i) bk.push_back(b.qshape[i + NB - K]);
  }
  c.q = a.q + b.q;
  for (int i = 0; i < K; ++i) {
    if (kq[i].size() != bk[i].size())
      throw Error(kQShapeMismatch, "btas::gemm_contract_qshape contraction of quantum numbers failed");
    for (size_t j = 0; j < kq[i].size(); ++j)
      if (kq[i][j] != -bk[i][j])
        throw Error(kQShapeMismatch, "btas::gemm_contract_qshape contraction of quantum numbers failed");
  }
  c.finalize();
  *Kout = K;
  return c;
}

namespace {
struct View {
  std::vector<std::pair<int64_t, int64_t>> ent;  // (view tag, original tag), ascending view tag
  std::vector<int64_t> shape;
};

// transposed_view(K): [i1..iK | iK+1..iN] -> [iK+1..iN | i1..iK]  (STArray.h:558-577)
View make_view(const Tensor& t, int K, bool transposed) {
  View v;
  const Shape& s = t.sh;
  const int N = s.rank;
  v.ent.reserve(t.tags.size());
  if (!transposed || K == N) {
    for (int64_t tg : t.tags) v.ent.emplace_back(tg, tg);
    for (int i = 0; i < N; ++i) v.shape.push_back(s.nsec(i));
    return v;
  }
  const int64_t oldstr = s.stride[K - 1];
  const int64_t newstr = s.nsparse / oldstr;
  for (int64_t tg : t.tags) v.ent.emplace_back(tg / oldstr + (tg % oldstr) * newstr, tg);
  std::sort(v.ent.begin(), v.ent.end());
  for (int i = K; i < N; ++i) v.shape.push_back(s.nsec(i));
  for (int i = 0; i < K; ++i) v.shape.push_back(s.nsec(i));
  return v;
}
}  // namespace

std::vector<GemmTaskRef> enumerate_gemm(Trans ta, Trans tb, const Tensor& a, const Tensor& b, const Shape& c,
                                        int K) {
  // QSTBLAS.h:215-225: NN -> (a, b^T view), NT -> (a, b), TN -> (a^T view, b^T view), TT -> (a^T view, b)
  const int L = a.sh.rank, M = b.sh.rank;
  View av = make_view(a, K, ta != kNoTrans);
  View bv = make_view(b, K, tb == kNoTrans);
  int64_t rowsA = 1, colsA = 1, colsB = 1;
  for (int i = 0; i < L - K; ++i) rowsA *= av.shape[i];
  for (int i = L - K; i < L; ++i) colsA *= av.shape[i];
  for (int i = 0; i < M - K; ++i) colsB *= bv.shape[i];
  (void)rowsA;
  // contiguous row ranges of the views
  auto rows_of = [&](const View& v) {
    std::vector<std::pair<int64_t, std::pair<size_t, size_t>>> r;
    size_t i = 0;
    while (i < v.ent.size()) {
      int64_t row = v.ent[i].first / colsA;
      size_t j = i;
      while (j < v.ent.size() && v.ent[j].first / colsA == row) ++j;
      r.push_back({row, {i, j}});
      i = j;
    }
    return r;
  };
  auto arows = rows_of(av);
  auto brows = rows_of(bv);
  std::vector<GemmTaskRef> tasks;
  for (auto& ar : arows) {
    const int64_t i = ar.first;
    for (auto& br : brows) {
      const int64_t j = br.first;
      const int64_t ij = i * colsB + j;
      if (!c.allowed_tag(ij)) continue;
      GemmTaskRef task;
      task.c_tag = ij;
      // pairs in (aik ascending, bjk ascending) order with equal contracted tag
      size_t pa = ar.second.first, pb = br.second.first;
      const size_t ea = ar.second.second, eb = br.second.second;
      while (pa < ea && pb < eb) {
        const int64_t ka = av.ent[pa].first % colsA;
        const int64_t kb = bv.ent[pb].first % colsA;
        if (ka == kb) {
          task.pairs.push_back({av.ent[pa].second, bv.ent[pb].second});
          ++pa;
          ++pb;
        } else if (ka < kb) {
          ++pa;
        } else {
          ++pb;
        }
      }
      if (!task.pairs.empty()) tasks.push_back(std::move(task));
    }
  }
  return tasks;
}

MergeInfo::MergeInfo(const std::vector<std::vector<Qn>>& qs, const std::vector<std::vector<int>>& ds)
    : qshape(qs), dshape(ds) {
  if (qs.size() != ds.size()) throw Error(kInvalidArgument, "merge info: qshape/dshape rank mismatch");
  q_packed.assign(1, Qn{});
  d_packed.assign(1, 1);
  for (size_t i = 0; i < qs.size(); ++i) {
    if (qs[i].size() != ds[i].size())
      throw Error(kInvalidArgument, "btas::QSTmergeInfo::reset: qshape and dshape have different block size");
    std::vector<Qn> nq;
    std::vector<int> nd;
    for (size_t x = 0; x < q_packed.size(); ++x)
      for (size_t y = 0; y < qs[i].size(); ++y) {
        nq.push_back(q_packed[x] + qs[i][y]);
        nd.push_back(d_packed[x] * ds[i][y]);
      }
    q_packed.swap(nq);
    d_packed.swap(nd);
  }
  std::map<std::pair<int, int>, int> order;
  for (const Qn& q : q_packed) {
    auto key = std::make_pair(q.p, q.s);
    if (!order.count(key)) {
      int n = static_cast<int>(order.size());
      order[key] = n;
    }
  }
  q_merged.assign(order.size(), Qn{});
  for (auto& kv : order) q_merged[kv.second] = Qn{kv.first.first, kv.first.second};
  d_merged.assign(order.size(), 0);
  members.assign(order.size(), {});
  merged_of.resize(q_packed.size());
  offset_packed.resize(q_packed.size());
  for (size_t i = 0; i < q_packed.size(); ++i) {
    const int j = order[std::make_pair(q_packed[i].p, q_packed[i].s)];
    merged_of[i] = j;
    offset_packed[i] = d_merged[j];
    members[j].push_back(static_cast<int>(i));
    d_merged[j] += d_packed[i];
  }
}

}  // namespace mpsxx
