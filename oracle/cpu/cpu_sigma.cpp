// CPU restatement of the reference's merged H_eff*psi on the BTAS block-sparse engine,
// for timing the reference's CPU algorithm on hosts where the reference itself cannot be
// built.  Oracle test infrastructure: only tests/ and bench.py's reference arm load it.
//
// Followed step by step (paths relative to the mpsxx tree):
//   * compute_sigma_vector, merged form (src/compute_sigma_vector.hpp:85-96): two Gemm's,
//     scr1[A,w,B'] = sum_A' L[A,w,A'] psi[A',B'] (K = 1), then
//     sigma[A,B]  = sum_{w,B'} scr1[A,w,B'] R[B,w,B'] (K = 2, right operand transposed);
//   * ST_Gemm_thread (include/btas/SPARSE/STBLAS.h:297-359): for each row block i of the
//     left operand and column block j of the right one whose result block is allowed, the
//     ordered (a_ik, b_jk) pairs with equal contracted tag; the right operand of an NN
//     product is walked through its transposed view (include/btas/SPARSE/STArray.h:558-577);
//   * parallel_call (include/btas/SPARSE/T_arguments.h:585-600): tasks sorted by the FLOPS_
//     proxy (sum over pairs of max(size a, size b), T_arguments.h:559-564), largest first,
//     OpenMP guided loop; each task accumulates its pairs serially into its own block with
//     a row-major dgemm (include/btas/DENSE/TBLAS.h:209-245), BLAS single-threaded.
// The BLAS is OpenBLAS opened at run time (scipy's bundled copy, "scipy_" prefix).
#include <dlfcn.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <string>
#include <vector>

namespace {

enum { kRowMajor = 101, kNoTrans = 111, kTrans = 112 };
using dgemm_t = void (*)(int, int, int, int, int, int, double, const double*, int, const double*, int, double,
                         double*, int);
using setthreads_t = void (*)(int);
dgemm_t g_dgemm = nullptr;
std::string g_error;
int g_default_threads = 1;

// A block-sparse tensor as the caller lays it out: sector counts and dims per index,
// stored tags ascending, each block's offset into one data array.
struct Tensor {
  int rank = 0;
  std::vector<int> nsec;                 // per index
  std::vector<std::vector<int>> dims;    // per index, per sector
  std::vector<int64_t> tags, offsets;    // ascending tags
  std::vector<int64_t> stride;           // row-major tag strides
  double* data = nullptr;
  std::vector<double> own;               // storage of results
  std::map<int64_t, int64_t> index;      // tag -> position

  void finish() {
    stride.assign(rank, 1);
    for (int i = rank - 2; i >= 0; --i) stride[i] = stride[i + 1] * nsec[i + 1];
    for (size_t k = 0; k < tags.size(); ++k) index[tags[k]] = static_cast<int64_t>(k);
  }
  int sector(int64_t tag, int i) const { return static_cast<int>((tag / stride[i]) % nsec[i]); }
  int64_t block_size(int64_t tag) const {
    int64_t s = 1;
    for (int i = 0; i < rank; ++i) s *= dims[i][sector(tag, i)];
    return s;
  }
  // rows/cols of a block viewed as a matrix with the first `nrow` indices as rows
  void matrix(int64_t tag, int nrow, int64_t& r, int64_t& c) const {
    r = c = 1;
    for (int i = 0; i < rank; ++i) (i < nrow ? r : c) *= dims[i][sector(tag, i)];
  }
};

struct Pair {
  int64_t a, b;  // positions in the operands' tag lists
};
struct Task {
  int64_t c;  // result tag
  std::vector<Pair> pairs;
  size_t flops_proxy = 0;
};

// ST_Gemm_thread over views: `av` / `bv` map view tags to stored positions; rowsA/colsA/colsB
// are the sparse extents of the views; `allowed(c_tag)` is the result's quantum rule.
std::vector<Task> enumerate(const std::vector<std::pair<int64_t, int64_t>>& av,
                            const std::vector<std::pair<int64_t, int64_t>>& bv, int64_t rowsA, int64_t colsA,
                            int64_t colsB, const std::function<bool(int64_t)>& allowed,
                            const std::function<size_t(int64_t, int64_t)>& proxy) {
  std::vector<Task> tasks;
  // rows of the (sorted) views
  auto row_ranges = [&](const std::vector<std::pair<int64_t, int64_t>>& v) {
    std::map<int64_t, std::pair<size_t, size_t>> r;
    for (size_t k = 0; k < v.size(); ++k) {
      const int64_t row = v[k].first / colsA;
      auto it = r.find(row);
      if (it == r.end())
        r[row] = {k, k + 1};
      else
        it->second.second = k + 1;
    }
    return r;
  };
  const auto ar = row_ranges(av), br = row_ranges(bv);
  for (const auto& ra : ar) {
    const int64_t i = ra.first;
    if (i >= rowsA) break;
    for (const auto& rb : br) {
      const int64_t j = rb.first;
      const int64_t ij = i * colsB + j;
      if (!allowed(ij)) continue;
      Task t;
      t.c = ij;
      for (size_t x = ra.second.first; x < ra.second.second; ++x)
        for (size_t y = rb.second.first; y < rb.second.second; ++y)
          if (av[x].first % colsA == bv[y].first % colsA) {
            t.pairs.push_back({av[x].second, bv[y].second});
            t.flops_proxy += proxy(av[x].second, bv[y].second);
          }
      if (!t.pairs.empty()) tasks.push_back(std::move(t));
    }
  }
  return tasks;
}

void run_tasks(std::vector<Task>& tasks, const std::function<void(const Task&)>& body) {
  std::sort(tasks.begin(), tasks.end(), [](const Task& x, const Task& y) { return x.flops_proxy > y.flops_proxy; });
  const int64_t n = static_cast<int64_t>(tasks.size());
#pragma omp parallel for schedule(guided)
  for (int64_t i = 0; i < n; ++i) body(tasks[i]);
}

// q-rule of a result block: sum of the sector quantum numbers of every index == total
struct QRule {
  std::vector<std::vector<std::pair<int, int>>> q;  // per index, per sector
  std::pair<int, int> total;
  std::vector<int64_t> stride;
  bool operator()(int64_t tag) const {
    int p = 0, s = 0;
    for (size_t i = 0; i < q.size(); ++i) {
      const auto& v = q[i][(tag / stride[i]) % q[i].size()];
      p += v.first;
      s += v.second;
    }
    return p == total.first && s == total.second;
  }
};

}  // namespace

extern "C" {

// Opens the BLAS (its cblas_dgemm under a scipy_ prefix or plain) and fixes its own
// threading to one; OpenMP runs the tasks on `threads` threads (<= 0: all).
int cpu_sigma_init(const char* blas_path, int threads) {
  void* h = dlopen(blas_path, RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    g_error = dlerror();
    return 1;
  }
  g_dgemm = reinterpret_cast<dgemm_t>(dlsym(h, "scipy_cblas_dgemm"));
  if (!g_dgemm) g_dgemm = reinterpret_cast<dgemm_t>(dlsym(h, "cblas_dgemm"));
  auto st = reinterpret_cast<setthreads_t>(dlsym(h, "scipy_openblas_set_num_threads"));
  if (!st) st = reinterpret_cast<setthreads_t>(dlsym(h, "openblas_set_num_threads"));
  if (!g_dgemm) {
    g_error = "no cblas_dgemm in the BLAS library";
    return 2;
  }
  if (st) st(1);
  g_default_threads = omp_get_max_threads();
  if (threads > 0) omp_set_num_threads(threads);
  return 0;
}

// OpenMP threads of the following runs: n > 0 threads, n <= 0 the count the process
// started with (OMP_NUM_THREADS or all cores).
void cpu_sigma_set_threads(int n) { omp_set_num_threads(n > 0 ? n : g_default_threads); }

const char* cpu_sigma_error() { return g_error.c_str(); }

int cpu_sigma_threads() { return omp_get_max_threads(); }

// H_eff*psi.  Each tensor: rank, nsec[rank], dims (concatenated per index), quantum numbers
// (p, s pairs concatenated per index), total q, ntags, tags, offsets, data.  sigma is laid out
// by the caller (S_desc/S_tags/S_offs, psi's quantum shape); its values are overwritten.  Returns the FLOPs (sum of 2mnk over both
// task lists) and the seconds of the two Gemm's (planning included, as the reference re-plans
// every call).
int cpu_sigma_run(const int* L_desc, const int64_t* L_tags, const int64_t* L_offs, double* L_data,
                  const int* R_desc, const int64_t* R_tags, const int64_t* R_offs, double* R_data,
                  const int* P_desc, const int64_t* P_tags, const int64_t* P_offs, double* P_data,
                  const int* S_desc, const int64_t* S_tags, const int64_t* S_offs, double* sigma_data,
                  double* flops_out, double* seconds_out) {
  if (!g_dgemm) {
    g_error = "cpu_sigma_init was not called";
    return 3;
  }
  // desc: rank, nsec..., dims..., (p,s)..., qp, qs, ntags
  auto parse = [](const int* d, const int64_t* tags, const int64_t* offs, double* data, Tensor& t,
                  std::vector<std::vector<std::pair<int, int>>>& q, std::pair<int, int>& qt) {
    int k = 0;
    t.rank = d[k++];
    t.nsec.assign(d + k, d + k + t.rank);
    k += t.rank;
    t.dims.resize(t.rank);
    for (int i = 0; i < t.rank; ++i) {
      t.dims[i].assign(d + k, d + k + t.nsec[i]);
      k += t.nsec[i];
    }
    q.resize(t.rank);
    for (int i = 0; i < t.rank; ++i)
      for (int s = 0; s < t.nsec[i]; ++s, k += 2) q[i].push_back({d[k], d[k + 1]});
    qt = {d[k], d[k + 1]};
    k += 2;
    const int n = d[k];
    t.tags.assign(tags, tags + n);
    t.offsets.assign(offs, offs + n);
    t.data = data;
    t.finish();
  };
  Tensor L, R, P, G;
  std::vector<std::vector<std::pair<int, int>>> qL, qR, qP, qG;
  std::pair<int, int> tL, tR, tP, tG;
  parse(L_desc, L_tags, L_offs, L_data, L, qL, tL);
  parse(R_desc, R_tags, R_offs, R_data, R, qR, tR);
  parse(P_desc, P_tags, P_offs, P_data, P, qP, tP);
  parse(S_desc, S_tags, S_offs, sigma_data, G, qG, tG);
  if (L.rank != 3 || R.rank != 3 || P.rank != 2) {
    g_error = "cpu_sigma_run: ranks must be 3, 3, 2";
    return 4;
  }
  const auto t0 = std::chrono::steady_clock::now();
  double flops = 0.0;

  // ---- stage 1: scr1 = L x psi (NN, K = 1); psi through its transposed view [B' | A'] ----
  const int64_t nA = L.nsec[0], nW = L.nsec[1], nAp = L.nsec[2], nBp = P.nsec[1];
  std::vector<std::pair<int64_t, int64_t>> av, bv;
  for (size_t k = 0; k < L.tags.size(); ++k) av.push_back({L.tags[k], static_cast<int64_t>(k)});
  for (size_t k = 0; k < P.tags.size(); ++k) {
    const int64_t a = P.tags[k] / nBp, b = P.tags[k] % nBp;
    bv.push_back({b * P.nsec[0] + a, static_cast<int64_t>(k)});
  }
  std::sort(bv.begin(), bv.end());
  // scr1 quantum shape [A, w, B'] (gemm_contract_qshape): total = qL + qP
  QRule s1;
  s1.q = {qL[0], qL[1], qP[1]};
  s1.total = {tL.first + tP.first, tL.second + tP.second};
  s1.stride = {nW * nBp, nBp, 1};
  auto sizeL = [&](int64_t k) { return static_cast<size_t>(L.block_size(L.tags[k])); };
  auto sizeP = [&](int64_t k) { return static_cast<size_t>(P.block_size(P.tags[k])); };
  std::vector<Task> t1 = enumerate(av, bv, nA * nW, nAp, nBp, s1,
                                   [&](int64_t a, int64_t b) { return std::max(sizeL(a), sizeP(b)); });
  // allocate scr1 blocks (tag order)
  Tensor S;
  S.rank = 3;
  S.nsec = {static_cast<int>(nA), static_cast<int>(nW), static_cast<int>(nBp)};
  S.dims = {L.dims[0], L.dims[1], P.dims[1]};
  for (const auto& t : t1) S.tags.push_back(t.c);
  std::sort(S.tags.begin(), S.tags.end());
  S.finish();
  int64_t total = 0;
  for (int64_t tag : S.tags) {
    S.offsets.push_back(total);
    total += S.block_size(tag);
  }
  S.own.assign(static_cast<size_t>(total), 0.0);
  S.data = S.own.data();
  for (const auto& t : t1)
    for (const auto& p : t.pairs) {
      int64_t m, k, k2, n;
      L.matrix(L.tags[p.a], 2, m, k);
      P.matrix(P.tags[p.b], 1, k2, n);
      flops += 2.0 * m * n * k;
    }
  run_tasks(t1, [&](const Task& t) {
    double* c = S.data + S.offsets[S.index.at(t.c)];
    for (const auto& p : t.pairs) {
      int64_t m, k, k2, n;
      L.matrix(L.tags[p.a], 2, m, k);
      P.matrix(P.tags[p.b], 1, k2, n);
      g_dgemm(kRowMajor, kNoTrans, kNoTrans, static_cast<int>(m), static_cast<int>(n), static_cast<int>(k), 1.0,
              L.data + L.offsets[p.a], static_cast<int>(k), P.data + P.offsets[p.b], static_cast<int>(n), 1.0, c,
              static_cast<int>(n));
    }
  });

  // ---- stage 2: sigma = scr1 x R^T (NT, K = 2 over (w, B')); both operands as stored ----
  av.clear();
  bv.clear();
  for (size_t k = 0; k < S.tags.size(); ++k) av.push_back({S.tags[k], static_cast<int64_t>(k)});
  for (size_t k = 0; k < R.tags.size(); ++k) bv.push_back({R.tags[k], static_cast<int64_t>(k)});
  const int64_t nB = R.nsec[0];
  QRule s2;
  s2.q = qP;
  s2.total = tP;
  s2.stride = {P.nsec[1], 1};
  auto sizeS = [&](int64_t k) { return static_cast<size_t>(S.block_size(S.tags[k])); };
  auto sizeR = [&](int64_t k) { return static_cast<size_t>(R.block_size(R.tags[k])); };
  std::vector<Task> t2 = enumerate(av, bv, nA, nW * nBp, nB, s2,
                                   [&](int64_t a, int64_t b) { return std::max(sizeS(a), sizeR(b)); });
  const int64_t nnz = G.offsets.empty() ? 0 : G.offsets.back() + G.block_size(G.tags.back());
  std::fill(sigma_data, sigma_data + nnz, 0.0);
  for (const auto& t : t2)
    for (const auto& p : t.pairs) {
      int64_t m, k, n, k2;
      S.matrix(S.tags[p.a], 1, m, k);
      R.matrix(R.tags[p.b], 1, n, k2);
      flops += 2.0 * m * n * k;
    }
  int missing = 0;
  run_tasks(t2, [&](const Task& t) {
    auto it = G.index.find(t.c);
    if (it == G.index.end()) {
#pragma omp atomic
      ++missing;
      return;
    }
    double* c = sigma_data + G.offsets[it->second];
    for (const auto& p : t.pairs) {
      int64_t m, k, n, k2;
      S.matrix(S.tags[p.a], 1, m, k);
      R.matrix(R.tags[p.b], 1, n, k2);
      g_dgemm(kRowMajor, kNoTrans, kTrans, static_cast<int>(m), static_cast<int>(n), static_cast<int>(k), 1.0,
              S.data + S.offsets[p.a], static_cast<int>(k), R.data + R.offsets[p.b], static_cast<int>(k), 1.0, c,
              static_cast<int>(n));
    }
  });
  *seconds_out = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *flops_out = flops;
  if (missing) {
    g_error = "cpu_sigma_run: a sigma block outside the given layout";
    return 5;
  }
  return 0;
}

}  // extern "C"
