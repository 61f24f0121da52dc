// Device engine of the merged two-site DMRG hot path: plans built once per
// layout on the host, executed by the sm_103a kernels.
#include "engine.hpp"

#include <algorithm>
#include <array>
#include <atomic>
#include <exception>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>
#include <tuple>

#include "jacobi.hpp"

namespace mpsxx {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(kCuda, std::string(what) + ": " + cudaGetErrorString(e));
}

void solver_check(cusolverStatus_t s, const char* what) {
  if (s != CUSOLVER_STATUS_SUCCESS) throw Error(kSolver, std::string(what) + ": cusolver status " + std::to_string(s));
}

// ---------------------------------------------------------------------------
// device block cache
// ---------------------------------------------------------------------------
namespace {
// A released block remembers the stream of its last owner.  Taken again on the same
// stream it needs no synchronisation (stream order); taken on another stream, that
// stream waits for an event recorded on the old one at that moment (which covers the
// old owner's work).  Released blocks thus cost no driver calls.
struct CachedBlock {
  void* p;
  int device;
  cudaStream_t st;  // stream of the last owner; nullptr: idle (its context drained it)
};

class BlockCache {
 public:
  // Rounded allocation size: powers of two below 2 MiB, multiples of 2 MiB above.
  static size_t round(size_t bytes) {
    bytes = std::max<size_t>(bytes, 512);
    if (bytes < (size_t(2) << 20)) {
      size_t r = 512;
      while (r < bytes) r <<= 1;
      return r;
    }
    const size_t g = size_t(2) << 20;
    return (bytes + g - 1) / g * g;
  }

  void* get(size_t bytes, cudaStream_t st, size_t* got) {
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    const size_t want = round(bytes);
    {
      std::lock_guard<std::mutex> lk(mu_);
      // best fit among blocks of at most 5/4 of the request
      for (auto it = free_.lower_bound(want); it != free_.end() && it->first <= want + want / 4; ++it) {
        if (it->second.device != dev) continue;
        CachedBlock b = it->second;
        *got = it->first;
        cached_ -= it->first;
        free_.erase(it);
        if (b.st && b.st != st) {
          // under the lock: the old stream cannot be unregistered and destroyed meanwhile
          cudaEvent_t ev = nullptr;
          cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "block cache event");
          cuda_check(cudaEventRecord(ev, b.st), "block cache record");
          const cudaError_t e = cudaStreamWaitEvent(st, ev, 0);
          cudaEventDestroy(ev);
          cuda_check(e, "block cache wait");
        }
        return b.p;
      }
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      trim();  // give the cached blocks back and try once more
      e = cudaMalloc(&p, want);
      if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(kAlloc, std::string("device allocation of ") + std::to_string(want) + " bytes failed: " +
                                cudaGetErrorString(e));
      }
    }
    *got = want;
    return p;
  }

  void put(void* p, size_t bytes, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu_);
    // a stream that is no longer registered belonged to a context that drained it
    // before going away: the block is idle
    const bool live = live_.count(st) > 0;
    free_.emplace(bytes, CachedBlock{p, dev, live ? st : nullptr});
    cached_ += bytes;
  }

  void register_stream(cudaStream_t st) {
    std::lock_guard<std::mutex> lk(mu_);
    live_[st] += 1;
  }
  // the stream's owner has drained it: its cached blocks become idle
  void unregister_stream(cudaStream_t st) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = live_.find(st);
    if (it != live_.end() && --it->second == 0) {
      live_.erase(it);
      for (auto& kv : free_)
        if (kv.second.st == st) kv.second.st = nullptr;
    }
  }

  // Free every cached block (cudaFree waits for the device's queued work first).
  void trim() {
    std::multimap<size_t, CachedBlock> blocks;
    {
      std::lock_guard<std::mutex> lk(mu_);
      blocks.swap(free_);
      cached_ = 0;
    }
    for (auto& kv : blocks) cudaFree(kv.second.p);
  }

  size_t cached_bytes() {
    std::lock_guard<std::mutex> lk(mu_);
    return cached_;
  }

 private:
  std::mutex mu_;
  std::multimap<size_t, CachedBlock> free_;
  std::map<cudaStream_t, int> live_;  // streams of live contexts
  size_t cached_ = 0;
};

// Never destroyed: blocks may be released during static destruction, after the
// CUDA runtime has begun shutting down.
BlockCache& block_cache() {
  static BlockCache* c = new BlockCache;
  return *c;
}
}  // namespace

void trim_block_cache() { block_cache().trim(); }
void register_cache_stream(cudaStream_t st) { block_cache().register_stream(st); }
size_t block_cache_bytes() { return block_cache().cached_bytes(); }

void DevBuf::ensure(size_t bytes, cudaStream_t stream) {
  if (bytes <= cap && stream == st) return;
  release();
  size_t got = 0;
  p = block_cache().get(bytes, stream, &got);
  cap = got;
  st = stream;
}

void DevBuf::release() {
  if (p) block_cache().put(p, cap, st);
  p = nullptr;
  cap = 0;
}

namespace {
// Host-to-device uploads of small host arrays (plans, Ritz vectors) go through a
// pinned staging area: the data is copied into it and the device copy is queued
// asynchronously, so an upload costs a memcpy and a queued copy instead of the
// driver's staging of pageable memory (which serialises concurrent planning threads).
// Two halves alternate; a half is refilled only after the copies queued from it have
// run (an event on every stream that read from it).  One stager per device.
class Stager {
 public:
  static constexpr size_t kHalf = size_t(16) << 20;
  static constexpr size_t kMaxStaged = size_t(1) << 20;  // larger uploads are copied directly

  void upload(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return;
    std::lock_guard<std::mutex> lk(mu_);
    if (!buf_[0] && !failed_) {
      void* p = nullptr;
      if (cudaHostAlloc(&p, 2 * kHalf, cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        failed_ = true;  // no pinned memory: plain copies
      } else {
        buf_[0] = static_cast<char*>(p);
        buf_[1] = buf_[0] + kHalf;
      }
    }
    if (failed_ || bytes > kMaxStaged) {
      cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "upload");
      return;
    }
    const size_t need = (bytes + 15) & ~size_t(15);
    if (off_ + need > kHalf) switch_half();
    char* p = buf_[cur_] + off_;
    off_ += need;
    std::memcpy(p, src, bytes);
    cuda_check(cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, st), "staged upload");
    if (std::find(used_[cur_].begin(), used_[cur_].end(), st) == used_[cur_].end()) used_[cur_].push_back(st);
  }

  // a stream about to be destroyed (its work drained): no event is recorded on it
  void forget(cudaStream_t st) {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& u : used_) u.erase(std::remove(u.begin(), u.end(), st), u.end());
  }

 private:
  void switch_half() {
    for (cudaStream_t s : used_[cur_]) {
      cudaEvent_t ev = nullptr;
      cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "stager event");
      cuda_check(cudaEventRecord(ev, s), "stager record");
      done_[cur_].push_back(ev);
    }
    used_[cur_].clear();
    cur_ ^= 1;
    off_ = 0;
    for (cudaEvent_t ev : done_[cur_]) {
      cudaEventSynchronize(ev);
      cudaEventDestroy(ev);
    }
    done_[cur_].clear();
  }

  std::mutex mu_;
  char* buf_[2] = {nullptr, nullptr};
  bool failed_ = false;
  int cur_ = 0;
  size_t off_ = 0;
  std::vector<cudaStream_t> used_[2];
  std::vector<cudaEvent_t> done_[2];
};

constexpr int kMaxDevices = 64;

// Never destroyed (uploads may be queued during static destruction).
Stager& stager() {
  static Stager* s = new Stager[kMaxDevices];
  int dev = 0;
  cudaGetDevice(&dev);
  return s[dev >= 0 && dev < kMaxDevices ? dev : 0];
}
}  // namespace

void upload_staged(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  stager().upload(dst, src, bytes, st);
}

void forget_stream_uploads(cudaStream_t st) {
  stager().forget(st);
}

template <class T>
void DevArray<T>::upload(const std::vector<T>& h, cudaStream_t st) {
  n = h.size();
  buf.ensure(std::max<size_t>(1, n) * sizeof(T), st);
  if (n) upload_staged(buf.p, h.data(), n * sizeof(T), st);
}
template struct DevArray<DTile>;
template struct DevArray<DSvdBlock>;
template struct DevArray<DEigBlock>;
template struct DevArray<DPkPair>;
template struct DevArray<DPack>;
template struct DevArray<DReduce>;
template struct DevArray<DBatchProb>;
template struct DevArray<DGemmTask>;
template struct DevArray<DGemmPair>;
template struct DevArray<DDiagTask>;
template struct DevArray<DDiagPair>;
template struct DevArray<DCopy>;
template struct DevArray<DScatterDst>;
template struct DevArray<DScatterSrc>;
template struct DevArray<DNoise>;
template struct DevArray<double>;
template struct DevArray<int64_t>;
template struct DevArray<int>;

void DTensor::alloc_device(cudaStream_t st, bool zero) {
  store.ensure(std::max<int64_t>(nnz, 1) * sizeof(double), st);
  d = store.as<double>();
  data_version = next_data_version();
  if (zero && nnz) cuda_check(cudaMemsetAsync(d, 0, nnz * sizeof(double), st), "tensor zero");
}

Context::Context(int dev, cudaStream_t st) : device(dev) {
  cuda_check(cudaSetDevice(dev), "cudaSetDevice");
  if (st) {
    stream = st;
  } else {
    cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream create");
    own_stream = true;
  }
  solver_check(cusolverDnCreate(&solver), "cusolverDnCreate");
  solver_check(cusolverDnSetStream(solver, stream), "cusolverDnSetStream");
  block_cache().register_stream(stream);
}

Context::~Context() {
  // drain the stream and hand the context's buffers back while it is registered
  cudaStreamSynchronize(stream);
  sigma_plans.clear();
  diag_plans.clear();
  merge_plans.clear();
  renorm_plans.clear();
  for (DevBuf* b : {&scr1, &scr2, &work, &partial, &scalars, &svd_work, &svd_mats, &gemm_part, &err_flag,
                    &svd_gram, &svd_gram_work, &svd_ptrs})
    b->release();
  forget_stream_uploads(stream);
  for (auto& l : svd_lanes) {
    cudaStreamSynchronize(l->stream);
    forget_stream_uploads(l->stream);
    l->work.release();
    block_cache().unregister_stream(l->stream);
    if (l->solver) cusolverDnDestroy(l->solver);
    if (l->blas) cublasDestroy(l->blas);
    if (l->done) cudaEventDestroy(l->done);
    cudaStreamDestroy(l->stream);
  }
  if (svd_ready) cudaEventDestroy(svd_ready);
  block_cache().unregister_stream(stream);
  if (solver) cusolverDnDestroy(solver);
  if (solver_params) cusolverDnDestroyParams(solver_params);
  if (blas) cublasDestroy(blas);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

void Context::sync() { cuda_check(cudaStreamSynchronize(stream), "stream sync"); }

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// with profiling on, device work queued before the phase is drained first so that it
// is not counted in this phase
namespace {
thread_local bool tl_planning = false;  // this thread builds plans for a batched step
}

PhaseTimer::PhaseTimer(Context& c, int ph) : ctx(c), phase(ph), on(c.profile && !tl_planning) {
  if (on) {
    cudaStreamSynchronize(c.stream);
    t0 = now();
  }
}

void PhaseTimer::stop() {
  if (!open) return;
  open = false;
  if (!on) return;
  cudaStreamSynchronize(ctx.stream);
  dt = now() - t0;
  ctx.timers[phase] += dt;
}

// ---------------------------------------------------------------------------
// grouped GEMM plans
// ---------------------------------------------------------------------------
static int64_t prod(const int* d, int lo, int hi) {
  int64_t p = 1;
  for (int i = lo; i < hi; ++i) p *= d[i];
  return p;
}

struct CMap {
  int64_t off;
  int m, n, ldc;
};

// Output tiles of every task; the pair list of long tasks is split (split-K) so
// that a launch fills the GPU: the work of a tile ~ the sum of its pairs' k.
static void make_tiles(const GemmPlan& plan, int tile_m, int tile_n, std::vector<DTile>& tiles,
                       std::vector<DReduce>& reduce, int& nslots, int target_ctas = kTargetCtas) {
  tiles.clear();
  reduce.clear();
  nslots = 0;
  double total = 0.0;
  for (const auto& dt : plan.h_tasks) {
    double k = 0.0;
    for (int p = dt.p0; p < dt.p1; ++p) k += plan.h_pairs[p].k;
    total += double((dt.m + tile_m - 1) / tile_m) * ((dt.n + tile_n - 1) / tile_n) * k;
  }
  const double target = std::max(1.0, total / target_ctas);
  for (int ti = 0; ti < static_cast<int>(plan.h_tasks.size()); ++ti) {
    const DGemmTask& dt = plan.h_tasks[ti];
    double k = 0.0;
    for (int p = dt.p0; p < dt.p1; ++p) k += plan.h_pairs[p].k;
    const int npair = dt.p1 - dt.p0;
    int nchunk = static_cast<int>(std::min<double>(npair, std::floor(k / target)));
    if (nchunk < 2) nchunk = 1;
    // chunk boundaries with about equal k
    std::vector<int> bnd{dt.p0};
    if (nchunk > 1) {
      double acc = 0.0, step = k / nchunk;
      for (int p = dt.p0; p < dt.p1 && static_cast<int>(bnd.size()) < nchunk; ++p) {
        acc += plan.h_pairs[p].k;
        if (acc >= step * bnd.size() && p + 1 < dt.p1) bnd.push_back(p + 1);
      }
    }
    bnd.push_back(dt.p1);
    const int nc = static_cast<int>(bnd.size()) - 1;
    const int ntm = (dt.m + tile_m - 1) / tile_m, ntn = (dt.n + tile_n - 1) / tile_n;
    if (nc == 1) {
      for (int tm = 0; tm < ntm; ++tm)
        for (int tn = 0; tn < ntn; ++tn) tiles.push_back(DTile{ti, tm, tn, bnd[0], bnd[1], -1});
      continue;
    }
    // chunk-major: tiles over the same K range follow each other, so the CTAs that run
    // together share their A row panels and B column panels in L2
    const int slot0 = nslots;
    for (int tm = 0; tm < ntm; ++tm)
      for (int tn = 0; tn < ntn; ++tn) reduce.push_back(DReduce{ti, tm, tn, slot0 + (tm * ntn + tn) * nc, nc, 0});
    for (int ch = 0; ch < nc; ++ch)
      for (int tm = 0; tm < ntm; ++tm)
        for (int tn = 0; tn < ntn; ++tn)
          tiles.push_back(DTile{ti, tm, tn, bnd[ch], bnd[ch + 1], slot0 + (tm * ntn + tn) * nc + ch});
    nslots += ntm * ntn * nc;
  }
}

static void tile_tc(GemmPlan& plan, int target_ctas);

template <class F>
static void build_plan_impl(GemmPlan& plan, Trans ta, Trans tb, const Tensor& a, const Tensor& b, int K,
                            std::vector<GemmTaskRef>&& tasks, F cmap) {
  plan.ta = ta;
  plan.tb = tb;
  plan.K = K;
  plan.tasks = std::move(tasks);
  plan.h_tiles.clear();
  plan.h_tasks.clear();
  plan.h_pairs.clear();
  plan.pair_a_slot.clear();
  plan.pair_b_slot.clear();
  plan.task_ctag.clear();
  plan.h_reduce.clear();
  plan.flops = 0.0;
  plan.c_elems = 0;
  const int L = a.sh.rank, M = b.sh.rank;
  for (const auto& t : plan.tasks) {
    const CMap c = cmap(t.c_tag);
    DGemmTask dt;
    dt.c_off = c.off;
    dt.m = c.m;
    dt.n = c.n;
    dt.ldc = c.ldc;
    dt.p0 = static_cast<int>(plan.h_pairs.size());
    for (const auto& pr : t.pairs) {
      const int32_t as = a.find(pr.a_tag), bs = b.find(pr.b_tag);
      if (as < 0 || bs < 0) throw Error(kInternal, "gemm plan: operand block missing");
      int ad[kMaxRank], bd[kMaxRank];
      a.block_dims(as, ad);
      b.block_dims(bs, bd);
      int64_t ma, ka, lda, kb, nb, ldb;
      if (ta == kNoTrans) {
        ma = prod(ad, 0, L - K);
        ka = prod(ad, L - K, L);
        lda = ka;
      } else {
        ka = prod(ad, 0, K);
        ma = prod(ad, K, L);
        lda = ma;
      }
      if (tb == kNoTrans) {
        kb = prod(bd, 0, K);
        nb = prod(bd, K, M);
        ldb = nb;
      } else {
        nb = prod(bd, 0, M - K);
        kb = prod(bd, M - K, M);
        ldb = kb;
      }
      if (ma != c.m || nb != c.n || ka != kb) throw Error(kInternal, "gemm plan: inconsistent block dims");
      if (ka == 0 || ma == 0 || nb == 0) continue;
      DGemmPair p;
      p.a_off = a.offsets[as];
      p.b_off = b.offsets[bs];
      p.k = static_cast<int>(ka);
      p.lda = static_cast<int>(lda);
      p.ldb = static_cast<int>(ldb);
      p.pad = 0;
      plan.h_pairs.push_back(p);
      plan.pair_a_slot.push_back(as);
      plan.pair_b_slot.push_back(bs);
      plan.flops += 2.0 * double(ma) * double(nb) * double(ka);
    }
    dt.p1 = static_cast<int>(plan.h_pairs.size());
    if (dt.p1 == dt.p0) continue;
    plan.h_tasks.push_back(dt);
    plan.task_ctag.push_back(t.c_tag);
    plan.c_elems += int64_t(c.m) * c.n;
  }
  make_tiles(plan, kGemmTile, kGemmTile, plan.h_tiles, plan.h_reduce, plan.nslots);
  tile_tc(plan, kTargetCtas);
}

// Tensor-core (128 x 64) tiling of a plan's tasks with split-K chunks sized for about
// target_ctas tiles, heaviest first: the kernel is persistent (CTA c takes tiles c,
// c + #SM, ...), so this is a longest-processing-time-first balance.
static void tile_tc(GemmPlan& plan, int target_ctas) {
  make_tiles(plan, kTcTileM, kTcTileN, plan.h_tiles_tc, plan.h_reduce_tc, plan.nslots_tc, target_ctas);
  for (DTile& t : plan.h_tiles_tc) {
    t.h64 = tail64(plan.h_tasks[t.task].m, t.tm) ? 1 : 0;
    t.nt = tail_cols(plan.h_tasks[t.task].n, t.tn);
  }
  std::vector<std::pair<int64_t, int>> work(plan.h_tiles_tc.size());
  for (size_t i = 0; i < plan.h_tiles_tc.size(); ++i) {
    int64_t w = 0;
    for (int p = plan.h_tiles_tc[i].p0; p < plan.h_tiles_tc[i].p1; ++p)
      w += (plan.h_pairs[p].k + kPkTileK - 1) / kPkTileK;
    work[i] = {-w, static_cast<int>(i)};
  }
  std::stable_sort(work.begin(), work.end());
  std::vector<DTile> sorted(plan.h_tiles_tc.size());
  for (size_t i = 0; i < work.size(); ++i) sorted[i] = plan.h_tiles_tc[work[i].second];
  plan.h_tiles_tc.swap(sorted);
}

void build_gemm_plan(GemmPlan& plan, Trans ta, Trans tb, const Tensor& a, const Tensor& b, const Tensor& c, int K,
                     std::vector<GemmTaskRef>&& tasks) {
  const int L = a.sh.rank;
  build_plan_impl(plan, ta, tb, a, b, K, std::move(tasks), [&](int64_t ctag) {
    const int32_t cs = c.find(ctag);
    if (cs < 0) throw Error(kInternal, "gemm plan: result block missing from the result layout");
    int cd[kMaxRank];
    c.block_dims(cs, cd);
    CMap m;
    m.off = c.offsets[cs];
    m.m = static_cast<int>(prod(cd, 0, L - K));
    m.n = static_cast<int>(prod(cd, L - K, c.sh.rank));
    m.ldc = m.n;
    return m;
  });
}

void GemmPlan::upload(cudaStream_t st) {
  tiles.upload(h_tiles, st);
  dtasks.upload(h_tasks, st);
  pairs.upload(h_pairs, st);
  reduce.upload(h_reduce, st);
  tiles_tc.upload(h_tiles_tc, st);
  reduce_tc.upload(h_reduce_tc, st);
}


void GemmPlan::run(double alpha, const double* A, const double* B, double* C, double* partial,
                   cudaStream_t st) const {
  if (nslots > 0 && partial == nullptr) throw Error(kInternal, "gemm plan: split-K scratch missing");
  launch_gemm_f64(ta, tb, alpha, A, B, C, tiles.get(), static_cast<int>(h_tiles.size()), dtasks.get(), pairs.get(),
                  partial, st);
  if (nslots > 0)
    launch_gemm_reduce(reduce.get(), static_cast<int>(h_reduce.size()), dtasks.get(), alpha, partial, C, st);
}

static double* gemm_scratch(Context& ctx, const GemmPlan& p) {
  if (p.nslots == 0) return nullptr;
  ctx.gemm_part.ensure(p.partial_bytes(), ctx.stream);
  return ctx.gemm_part.as<double>();
}

// Result tensor whose blocks are exactly the task results (a Gemm into an empty array).
static void layout_from_tasks(Tensor& c, const Shape& sh, const std::vector<GemmTaskRef>& tasks) {
  c.sh = sh;
  std::vector<int64_t> t;
  t.reserve(tasks.size());
  for (const auto& x : tasks) t.push_back(x.c_tag);
  std::sort(t.begin(), t.end());
  c.set_blocks(t);
}

static Tensor conj_view(const Tensor& t) {
  Tensor c;
  c.sh = t.sh.conjugate();
  c.tags = t.tags;
  c.offsets = t.offsets;
  c.slot = t.slot;
  c.nnz = t.nnz;
  c.d = t.d;
  c.layout_id = t.layout_id;
  return c;
}

static bool same_qshape(const Shape& a, const Shape& b) {
  if (a.rank != b.rank || a.q != b.q) return false;
  for (int i = 0; i < a.rank; ++i) {
    if (a.qshape[i].size() != b.qshape[i].size()) return false;
    for (size_t j = 0; j < a.qshape[i].size(); ++j)
      if (a.qshape[i][j] != b.qshape[i][j]) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// plan caches (shared with planning threads)
// ---------------------------------------------------------------------------
template <class M, class K>
static typename M::mapped_type::element_type* find_plan(Context& ctx, M& m, const K& key) {
  std::lock_guard<std::mutex> lk(ctx.plan_mu);
  auto it = m.find(key);
  return it == m.end() ? nullptr : it->second.get();
}

// Inserts a freshly built plan, or returns the one another planning thread inserted
// first.  A full cache is emptied first, except while planning threads hold
// references into it.
template <class M, class K, class P>
static P& insert_plan(Context& ctx, M& m, const K& key, std::unique_ptr<P> p) {
  std::lock_guard<std::mutex> lk(ctx.plan_mu);
  auto it = m.find(key);
  if (it != m.end()) return *it->second;
  if (m.size() >= ctx.max_plans && !ctx.planning_threads) m.clear();
  return *m.emplace(key, std::move(p)).first->second;
}

void reserve_plans(Context& ctx, size_t n) {
  std::lock_guard<std::mutex> lk(ctx.plan_mu);
  if (ctx.sigma_plans.size() + n > ctx.max_plans) ctx.sigma_plans.clear();
  if (ctx.diag_plans.size() + n > ctx.max_plans) ctx.diag_plans.clear();
  if (ctx.merge_plans.size() + 2 * n > ctx.max_plans) ctx.merge_plans.clear();
  if (ctx.renorm_plans.size() + n > ctx.max_plans) ctx.renorm_plans.clear();
}

void parallel_plan(Context& ctx, int n, const std::function<void(int)>& f) {
  const int hw = std::max(1, static_cast<int>(std::thread::hardware_concurrency()));
  const int nt = std::min({n, hw, 16});
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  ctx.planning_threads = true;
  std::atomic<int> next{0};
  std::vector<std::exception_ptr> errs(nt);
  auto work = [&](int t) {
    tl_planning = true;
    try {
      cuda_check(cudaSetDevice(ctx.device), "cudaSetDevice");
      for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) f(i);
    } catch (...) {
      errs[t] = std::current_exception();
    }
    tl_planning = false;
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  ctx.planning_threads = false;
  for (auto& e : errs)
    if (e) std::rethrow_exception(e);
}

// ---------------------------------------------------------------------------
// sigma vector
// ---------------------------------------------------------------------------
SigmaPlan& sigma_plan(Context& ctx, const Tensor& L, const Tensor& R, const Tensor& psi) {
  auto key = std::make_tuple(L.layout_id, R.layout_id, psi.layout_id);
  if (SigmaPlan* hit = find_plan(ctx, ctx.sigma_plans, key)) return *hit;
  PhaseTimer tm(ctx, kPhSigmaPlan);
  if (L.sh.rank != 3 || R.sh.rank != 3 || psi.sh.rank != 2)
    throw Error(kInvalidArgument, "compute_sigma_vector: expects 3-index operators and a 2-index wavefunction");
  auto p = std::make_unique<SigmaPlan>();
  p->l_id = L.layout_id;
  p->r_id = R.layout_id;
  p->psi_id = psi.layout_id;
  int K1 = 0, K2 = 0;
  Shape s1 = gemm_result_shape(kNoTrans, kNoTrans, L.sh, psi.sh, 3, &K1);
  auto t1 = enumerate_gemm(kNoTrans, kNoTrans, L, psi, s1, K1);
  layout_from_tasks(p->scr1, s1, t1);
  Shape s2 = gemm_result_shape(kNoTrans, kTrans, s1, R.sh, 2, &K2);
  if (!same_qshape(s2, psi.sh))
    throw Error(kQShapeMismatch, "Gemm(QSPARSE): c must have the same quantum shape of [ a * b ].");
  auto t2 = enumerate_gemm(kNoTrans, kTrans, p->scr1, R, s2, K2);
  build_gemm_plan(p->s1, kNoTrans, kNoTrans, L, psi, p->scr1, K1, std::move(t1));
  build_gemm_plan(p->s2, kNoTrans, kTrans, p->scr1, R, psi, K2, std::move(t2));
  p->s1.upload(ctx.stream);
  p->s2.upload(ctx.stream);
  p->flops = p->s1.flops + p->s2.flops;
  p->bytes_min = 8 * (L.nnz + R.nnz + 2 * psi.nnz);
  p->psi_layout = psi;
  p->psi_layout.d = nullptr;
  p->ops_single = ctx.sigma_fp32_operators;
  return insert_plan(ctx, ctx.sigma_plans, key, std::move(p));
}

// ---------------------------------------------------------------------------
// split-TF32 sigma over pre-packed operands
// ---------------------------------------------------------------------------
// Orientation of block b of a tensor as a GEMM operand: rows (A rows or B^T rows),
// K, leading dimension and whether the stored block is K-major (trans = 0) or
// rows-major along K (trans = 1).
struct Orient {
  int rows, k, ld, trans;
};

// Packed tile grid of an operand: per block, row tiles x K slices, row tile tr slice tk
// at base + (tr * nks + tk) * tile_bytes.  Tensor-core operands (128-row tiles) end in
// a compact tile: A operands (role 'A') in a 64-row tile where tail64 says so, B
// operands (role 'B') in a tile of tail_cols rows; the compact tile's slices sit at
// base + tr * nks * tile_bytes + tk * (its bytes per slice).
template <class F>
static void packed_layout(Packed& P, const Tensor& t, int tile_rows, uint32_t tile_bytes, F orient, int fp32 = 0,
                          char role = 'A') {
  P.base.assign(t.tags.size(), -1);
  P.nks.assign(t.tags.size(), 0);
  P.h_packs.clear();
  const bool tailed = tile_rows == 128;
  int64_t off = 0;
  // rows of row tile tr of a block of `rows` rows
  auto rows_of = [&](int rows, int tr) {
    if (!tailed) return tile_rows;
    if (role == 'B') return tail_cols(rows, tr);
    return tail64(rows, tr) ? 64 : tile_rows;
  };
  for (size_t b = 0; b < t.tags.size(); ++b) {
    const Orient o = orient(static_cast<int32_t>(b));
    if (o.rows <= 0 || o.k <= 0) continue;
    const int ntr = (o.rows + tile_rows - 1) / tile_rows;
    const int nks = (o.k + kPkTileK - 1) / kPkTileK;
    P.base[b] = off;
    P.nks[b] = nks;
    for (int tr = 0; tr < ntr; ++tr) {
      const int rt = rows_of(o.rows, tr);
      const int64_t slice = int64_t(tile_bytes) * rt / tile_rows;
      for (int tk = 0; tk < nks; ++tk)
        P.h_packs.push_back(DPack{t.offsets[b], off + int64_t(tr) * nks * tile_bytes + int64_t(tk) * slice, o.rows,
                                  o.k, o.ld, o.trans, rt, tr * tile_rows, tk, fp32, 0, rt});
    }
    const int rl = rows_of(o.rows, ntr - 1);
    off += int64_t(ntr - 1) * nks * tile_bytes + int64_t(nks) * (int64_t(tile_bytes) * rl / tile_rows);
  }
  P.bytes = off;
}

// Stacked stage 1 (see SigmaPlan::stack1).  Each stage-1 task (an L*psi block) has a
// single pair (L block, psi block); the tasks sharing a psi block form a panel whose
// rows are their L blocks' rows in task order, packed as 128-row A tiles (a last tile
// of at most 64 rows compact, as everywhere).  One pair per panel, one tile per
// (panel row tile, psi column tile), and a row map from panel rows to output rows.
static void build_stacked_stage1(Context& ctx, SigmaPlan& p, const Tensor& L) {
  const GemmPlan& g = p.s1;
  const uint32_t tile_bytes = p.ops_single ? kPkTileA1Bytes : kPkTileABytes;
  const int fp32 = p.ops_single ? 1 : 0;
  // panels: psi block slot -> tasks in task order
  std::map<int32_t, std::vector<int>> panels;
  for (size_t ti = 0; ti < g.h_tasks.size(); ++ti) {
    const DGemmTask& t = g.h_tasks[ti];
    if (t.p1 - t.p0 != 1) throw Error(kInternal, "stacked stage 1: a task with more than one pair");
    panels[g.pair_b_slot[t.p0]].push_back(static_cast<int>(ti));
  }
  Packed& P = p.pk_L;
  P.base.assign(L.tags.size(), -1);
  P.nks.assign(L.tags.size(), 0);
  P.h_packs.clear();
  p.h_stpk1.clear();
  p.h_row_map.clear();
  std::vector<DTile> tiles;
  int64_t off = 0;
  for (const auto& kv : panels) {
    const std::vector<int>& tk = kv.second;
    const DGemmPair& pr0 = g.h_pairs[g.h_tasks[tk[0]].p0];
    const int K = pr0.k, n = g.h_tasks[tk[0]].n;
    const int nks = (K + kPkTileK - 1) / kPkTileK;
    int64_t rows = 0;
    for (int ti : tk) {
      const DGemmTask& t = g.h_tasks[ti];
      if (g.h_pairs[t.p0].k != K || t.n != n) throw Error(kInternal, "stacked stage 1: panel shapes differ");
      rows += t.m;
    }
    if (rows > (int64_t(1) << 30)) throw Error(kInternal, "stacked stage 1: panel too tall");
    const int R = static_cast<int>(rows);
    const int ntr = (R + kTcTileM - 1) / kTcTileM;
    const int64_t map0 = static_cast<int64_t>(p.h_row_map.size());
    // row map: panel rows in task order, then padding up to the last tile's rows
    for (int ti : tk)
      for (int r = 0; r < g.h_tasks[ti].m; ++r) p.h_row_map.push_back((int64_t(ti) << 32) | int64_t(r));
    const int padded = (ntr - 1) * kTcTileM + (tail64(R, ntr - 1) ? 64 : kTcTileM);
    for (int r = R; r < padded; ++r) p.h_row_map.push_back(-1);
    // packs: for every row tile and K slice, one pack per block segment of the tile
    // (the tile's last segment also zero-fills the rows after it)
    const int64_t base = off;
    size_t j0 = 0;   // first task overlapping the current row tile
    int prow0 = 0;   // its first panel row
    for (int tr = 0; tr < ntr; ++tr) {
      const int rt = tail64(R, tr) ? 64 : kTcTileM;
      const int64_t slice = int64_t(tile_bytes) * rt / kTcTileM;
      const int row0 = tr * kTcTileM;
      while (j0 < tk.size() && prow0 + g.h_tasks[tk[j0]].m <= row0) prow0 += g.h_tasks[tk[j0++]].m;
      for (int ks = 0; ks < nks; ++ks) {
        const int64_t dst = base + int64_t(tr) * nks * tile_bytes + int64_t(ks) * slice;
        int prow = prow0;
        for (size_t j = j0; j < tk.size(); ++j) {
          const DGemmTask& t = g.h_tasks[tk[j]];
          const int lo = std::max(prow, row0), hi = std::min(prow + t.m, row0 + rt);
          const bool last = (prow + t.m >= row0 + rt) || j + 1 == tk.size();
          if (lo < hi || last) {
            const int32_t as = g.pair_a_slot[t.p0];
            const int span = last ? row0 + rt - lo : hi - lo;
            int d[kMaxRank];
            L.block_dims(as, d);
            P.h_packs.push_back(DPack{L.offsets[as], dst, d[0] * d[1], d[2], d[2], 0, rt, lo - prow, ks, fp32,
                                      lo - row0, span});
          }
          if (last) break;
          prow += t.m;
        }
      }
    }
    off += int64_t(ntr - 1) * nks * tile_bytes + int64_t(nks) * (int64_t(tile_bytes) * (tail64(R, ntr - 1) ? 64 : kTcTileM) / kTcTileM);
    const int panel = static_cast<int>(p.h_stpk1.size());
    const int32_t bs = g.pair_b_slot[g.h_tasks[tk[0]].p0];
    if (p.pk_psi.base[bs] < 0 || p.pk_psi.nks[bs] != nks) throw Error(kInternal, "stacked stage 1: psi packing mismatch");
    if (map0 > 0x7fffffff) throw Error(kInternal, "stacked stage 1: row map too large");
    p.h_stpk1.push_back(DPkPair{base, p.pk_psi.base[bs], nks, static_cast<int>(map0)});
    for (int tr = 0; tr < ntr; ++tr)
      for (int tn = 0; tn * kTcTileN < n; ++tn)
        tiles.push_back(DTile{tk[0], tr, tn, panel, panel + 1, -1, tail64(R, tr) ? 1 : 0, tail_cols(n, tn)});
  }
  P.bytes = off;
  // heaviest first (persistent CTAs take tiles round-robin)
  std::stable_sort(tiles.begin(), tiles.end(), [&](const DTile& a, const DTile& b) {
    return p.h_stpk1[a.p0].nks > p.h_stpk1[b.p0].nks;
  });
  p.h_st1 = std::move(tiles);
  p.st1.upload(p.h_st1, ctx.stream);
  p.stpk1.upload(p.h_stpk1, ctx.stream);
  p.row_map.upload(p.h_row_map, ctx.stream);
}

static void build_sigma_pk(Context& ctx, SigmaPlan& p, const Tensor& L, const Tensor& R, const Tensor& psi) {
  auto dims3 = [](const Tensor& t, int32_t b, int* d) { t.block_dims(b, d); };
  // stage 1: A = L block (dA x dA'), B^T = psi block transposed (dB' x dA'); the
  // operators as FP32 tiles (split on chip) or as hi|lo tiles
  packed_layout(p.pk_L, L, kTcTileM, p.ops_single ? kPkTileA1Bytes : kPkTileABytes, [&](int32_t b) {
    int d[kMaxRank];
    dims3(L, b, d);
    return Orient{d[0] * d[1], d[2], d[2], 0};
  }, p.ops_single ? 1 : 0);
  packed_layout(p.pk_psi, psi, kTcTileN, kPkTileBBytes, [&](int32_t b) {
    int d[kMaxRank];
    dims3(psi, b, d);
    return Orient{d[1], d[0], d[1], 1};
  }, 0, 'B');
  // stage-1 output = stage-2 A operand: scr1 block (dA x dB')
  // written by stage 1 and read once by stage 2: hi|lo tiles, or FP32 tiles split on chip
  packed_layout(p.pk_scr1, p.scr1, kTcTileM, p.scr1_single ? kPkTileA1Bytes : kPkTileABytes, [&](int32_t b) {
    int d[kMaxRank];
    dims3(p.scr1, b, d);
    return Orient{d[0] * d[1], d[2], d[2], 0};
  });
  // stage 2: B^T = R block (dB x dB')
  packed_layout(p.pk_R, R, kTcTileN, p.ops_single ? kPkTileB1Bytes : kPkTileBBytes, [&](int32_t b) {
    int d[kMaxRank];
    dims3(R, b, d);
    return Orient{d[0] * d[1], d[2], d[2], 0};
  }, p.ops_single ? 1 : 0, 'B');
  auto pairs_of = [](const GemmPlan& g, const Packed& A, const Packed& B, std::vector<DPkPair>& out) {
    out.resize(g.h_pairs.size());
    for (size_t i = 0; i < g.h_pairs.size(); ++i) {
      const int32_t as = g.pair_a_slot[i], bs = g.pair_b_slot[i];
      if (A.base[as] < 0 || B.base[bs] < 0 || A.nks[as] != B.nks[bs])
        throw Error(kInternal, "packed sigma plan: operand packing mismatch");
      out[i] = DPkPair{A.base[as], B.base[bs], A.nks[as], 0};
    }
  };
  // Stacked stage 1 where the schedule allows it (whole-w passes; w groups and batched
  // steps address L block by block): replaces the per-block packing of L
  const bool was_stacked = p.stack1;
  p.stack1 = p.allow_stack && ctx.sigma_w_budget <= 0 && p.pk_scr1.bytes <= kGroupIntermediateBytes;
  if (p.stack1 != was_stacked) p.pk_L.src_version = ~0ull;  // its packed contents follow the other layout
  if (p.stack1) build_stacked_stage1(ctx, p, L);
  else pairs_of(p.s1, p.pk_L, p.pk_psi, p.h_pk1);
  pairs_of(p.s2, p.pk_scr1, p.pk_R, p.h_pk2);
  // Stage 1 writes each tile's result straight into the intermediate's packed tiles,
  // which is right only for a tile summed in one piece: not split along K, one
  // accumulation group (psi has one block per column sector, so each L*psi block has
  // a single contributing pair)
  for (const DTile& t : p.s1.h_tiles_tc) {
    if (p.stack1) break;  // stacked tiles have one pair by construction
    int64_t kpad = 0;
    for (int q = t.p0; q + 1 < t.p1; ++q) kpad += int64_t(p.h_pk1[q].nks) * kPkTileK;
    if (t.slot >= 0 || kpad >= kFlushK)
      throw Error(kInternal, "packed sigma plan: a stage-1 tile is not summed in one piece");
  }
  // stage-1 tasks write packed scr1: c_off = byte base of the block, ldc = its K slices
  p.h_pk_tasks1 = p.s1.h_tasks;
  for (size_t ti = 0; ti < p.h_pk_tasks1.size(); ++ti) {
    const int32_t cs = p.scr1.find(p.s1.task_ctag[ti]);
    if (cs < 0 || p.pk_scr1.base[cs] < 0) throw Error(kInternal, "packed sigma plan: stage-1 output missing");
    p.h_pk_tasks1[ti].c_off = p.pk_scr1.base[cs];
    p.h_pk_tasks1[ti].ldc = p.pk_scr1.nks[cs];
  }
  if (!p.stack1) p.pk1.upload(p.h_pk1, ctx.stream);
  p.pk2.upload(p.h_pk2, ctx.stream);
  p.pk_tasks1.upload(p.h_pk_tasks1, ctx.stream);
  p.pk_L.packs.upload(p.pk_L.h_packs, ctx.stream);
  p.pk_R.packs.upload(p.pk_R.h_packs, ctx.stream);
  p.pk_psi.packs.upload(p.pk_psi.h_packs, ctx.stream);
  p.pk_built = true;
}

static void pack_into(Context& ctx, Packed& P, const DTensor& t) {
  launch_pack(P.packs.get(), static_cast<int>(P.h_packs.size()), t.d, P.buf.as<uint8_t>(), ctx.stream);
  P.src_layout = t.layout_id;
  P.src_version = t.data_version;
  ctx.kernel_launches += 1;
}

static void build_split_gemm(Context& ctx, SplitGemm& sg, const GemmPlan& g, const Tensor& a, const Tensor& b) {
  // operand orientation from the plan: A tiles hold rows m with K inner, B tiles rows n
  std::vector<Orient> oa(a.tags.size(), Orient{0, 0, 0, 0}), ob(b.tags.size(), Orient{0, 0, 0, 0});
  for (size_t t = 0; t < g.h_tasks.size(); ++t) {
    const DGemmTask& tk = g.h_tasks[t];
    for (int p = tk.p0; p < tk.p1; ++p) {
      const DGemmPair& pr = g.h_pairs[p];
      oa[g.pair_a_slot[p]] = Orient{tk.m, pr.k, pr.lda, g.ta == kTrans ? 1 : 0};
      ob[g.pair_b_slot[p]] = Orient{tk.n, pr.k, pr.ldb, g.tb == kTrans ? 0 : 1};
    }
  }
  packed_layout(sg.pa, a, kTcTileM, kPkTileABytes, [&](int32_t s) { return oa[s]; });
  packed_layout(sg.pb, b, kTcTileN, kPkTileBBytes, [&](int32_t s) { return ob[s]; }, 0, 'B');
  sg.h_pk.resize(g.h_pairs.size());
  for (size_t i = 0; i < g.h_pairs.size(); ++i) {
    const int32_t as = g.pair_a_slot[i], bs = g.pair_b_slot[i];
    if (sg.pa.base[as] < 0 || sg.pb.base[bs] < 0 || sg.pa.nks[as] != sg.pb.nks[bs])
      throw Error(kInternal, "split gemm plan: operand packing mismatch");
    sg.h_pk[i] = DPkPair{sg.pa.base[as], sg.pb.base[bs], sg.pa.nks[as], 0};
  }
  sg.pk.upload(sg.h_pk, ctx.stream);
  sg.pa.packs.upload(sg.pa.h_packs, ctx.stream);
  sg.pb.packs.upload(sg.pb.h_packs, ctx.stream);
}

// C += alpha * op(A) op(B) over the plan's tasks, in split TF32 (g uploaded).
static void run_split_gemm(Context& ctx, SplitGemm& sg, const GemmPlan& g, double alpha, const double* A,
                           const double* B, double* C) {
  if (g.h_tasks.empty()) return;
  sg.pa.buf.ensure(std::max<int64_t>(sg.pa.bytes, 16), ctx.stream);
  sg.pb.buf.ensure(std::max<int64_t>(sg.pb.bytes, 16), ctx.stream);
  launch_pack(sg.pa.packs.get(), static_cast<int>(sg.pa.h_packs.size()), A, sg.pa.buf.as<uint8_t>(), ctx.stream);
  launch_pack(sg.pb.packs.get(), static_cast<int>(sg.pb.h_packs.size()), B, sg.pb.buf.as<uint8_t>(), ctx.stream);
  ctx.gemm_part.ensure(std::max<size_t>(g.partial_bytes_tc(), 16), ctx.stream);
  double* part = ctx.gemm_part.as<double>();
  int* err = device_err_flag(ctx);
  launch_gemm_pk(sg.pa.buf.as<uint8_t>(), sg.pb.buf.as<uint8_t>(), alpha, C, nullptr, g.tiles_tc.get(),
                 static_cast<int>(g.h_tiles_tc.size()), g.dtasks.get(), sg.pk.get(), part, kOutFP64, 0, err,
                 ctx.stream, ctx.device_timeout_ns);
  if (g.nslots_tc > 0)
    launch_gemm_pk_reduce(g.reduce_tc.get(), static_cast<int>(g.h_reduce_tc.size()), g.dtasks.get(), alpha, part, C,
                          ctx.stream);
  ctx.kernel_launches += 3 + (g.nslots_tc > 0);
}

// w-groups of a sigma plan for a scratch budget (bytes of packed L*psi per group).
static void build_sigma_groups(Context& ctx, SigmaPlan& p, int64_t budget) {
  p.groups.clear();
  p.group_scr_bytes = 0;
  p.group_slots = 0;
  const Tensor& s = p.scr1;
  const int nw = s.sh.nsec(1);
  // packed bytes of every L*psi block and its w
  std::vector<int64_t> blk_bytes(s.tags.size(), 0), w_bytes(nw, 0);
  std::vector<int> blk_w(s.tags.size(), 0);
  for (size_t b = 0; b < s.tags.size(); ++b) {
    int d[kMaxRank], idx[kMaxRank];
    s.block_dims(static_cast<int32_t>(b), d);
    s.sh.index(s.tags[b], idx);
    blk_w[b] = idx[1];
    if (p.pk_scr1.base[b] < 0) continue;
    const int rows = d[0] * d[1];
    const int64_t ntr = (rows + kTcTileM - 1) / kTcTileM;
    const int64_t tb = p.scr1_single ? kPkTileA1Bytes : kPkTileABytes;
    // as packed_layout: a compact 64-row tail tile takes half a tile's bytes
    blk_bytes[b] = (ntr - (tail64(rows, ntr - 1) ? 1 : 0)) * p.pk_scr1.nks[b] * tb +
                   (tail64(rows, ntr - 1) ? p.pk_scr1.nks[b] * (tb / 2) : 0);
    w_bytes[idx[1]] += blk_bytes[b];
  }
  std::vector<int> group_of_w(nw, 0);
  int ng = 0;
  int64_t cur = 0;
  for (int w = 0; w < nw; ++w) {
    if (w_bytes[w] == 0) {
      group_of_w[w] = std::max(ng - 1, 0);
      continue;
    }
    if (ng == 0 || (budget > 0 && cur > 0 && cur + w_bytes[w] > budget)) {
      ++ng;
      cur = 0;
    }
    group_of_w[w] = ng - 1;
    cur += w_bytes[w];
  }
  ng = std::max(ng, 1);
  // group-local packed bases of the L*psi blocks
  std::vector<int64_t> local(s.tags.size(), -1), fill(ng, 0);
  for (size_t b = 0; b < s.tags.size(); ++b) {
    if (blk_bytes[b] == 0) continue;
    const int g = group_of_w[blk_w[b]];
    local[b] = fill[g];
    fill[g] += blk_bytes[b];
  }
  for (int g = 0; g < ng; ++g) p.group_scr_bytes = std::max(p.group_scr_bytes, fill[g]);
  // stage 1: tasks rebased, tiles bucketed by group
  std::vector<DGemmTask> tasks1 = p.h_pk_tasks1;
  std::vector<int> task1_group(tasks1.size(), 0);
  for (size_t ti = 0; ti < tasks1.size(); ++ti) {
    const int32_t cs = s.find(p.s1.task_ctag[ti]);
    if (cs < 0 || local[cs] < 0) throw Error(kInternal, "grouped sigma plan: stage-1 output missing");
    tasks1[ti].c_off = local[cs];
    task1_group[ti] = group_of_w[blk_w[cs]];
  }
  std::vector<std::vector<DTile>> t1(ng), t2(ng);
  std::vector<std::vector<DReduce>> red(ng);
  std::vector<int> slots(ng, 0);
  for (const DTile& t : p.s1.h_tiles_tc) {
    if (t.slot >= 0) throw Error(kInternal, "grouped sigma plan: stage 1 is not split along K");
    t1[task1_group[t.task]].push_back(t);
  }
  // stage 2: pairs rebased; per task the runs of consecutive pairs in one group
  std::vector<DPkPair> pairs2 = p.h_pk2;
  std::vector<int> pair_group(pairs2.size(), 0);
  for (size_t i = 0; i < pairs2.size(); ++i) {
    const int32_t as = p.s2.pair_a_slot[i];
    pairs2[i].a_pk = local[as];
    pair_group[i] = group_of_w[blk_w[as]];
  }
  struct Run {
    int task, p0, p1;
    double k;
  };
  std::vector<std::vector<Run>> runs(ng);
  std::vector<double> gwork(ng, 0.0);
  for (int ti = 0; ti < static_cast<int>(p.s2.h_tasks.size()); ++ti) {
    const DGemmTask& dt = p.s2.h_tasks[ti];
    const double tiles = double((dt.m + kTcTileM - 1) / kTcTileM) * ((dt.n + kTcTileN - 1) / kTcTileN);
    for (int a = dt.p0; a < dt.p1;) {
      int b = a;
      double k = 0.0;
      while (b < dt.p1 && pair_group[b] == pair_group[a]) k += p.s2.h_pairs[b++].k;
      runs[pair_group[a]].push_back(Run{ti, a, b, k});
      gwork[pair_group[a]] += tiles * k;
      a = b;
    }
  }
  for (int g = 0; g < ng; ++g) {
    const double target = std::max(1.0, gwork[g] / kTargetCtas);
    for (const Run& r : runs[g]) {
      const DGemmTask& dt = p.s2.h_tasks[r.task];
      int nchunk = static_cast<int>(std::min<double>(r.p1 - r.p0, std::floor(r.k / target)));
      if (nchunk < 2) nchunk = 1;
      std::vector<int> bnd{r.p0};
      if (nchunk > 1) {
        double acc = 0.0, step = r.k / nchunk;
        for (int q = r.p0; q < r.p1 && static_cast<int>(bnd.size()) < nchunk; ++q) {
          acc += p.s2.h_pairs[q].k;
          if (acc >= step * bnd.size() && q + 1 < r.p1) bnd.push_back(q + 1);
        }
      }
      bnd.push_back(r.p1);
      const int nc = static_cast<int>(bnd.size()) - 1;
      for (int tm = 0; tm * kTcTileM < dt.m; ++tm)
        for (int tn = 0; tn * kTcTileN < dt.n; ++tn) {
          if (nc == 1) {
            t2[g].push_back(DTile{r.task, tm, tn, bnd[0], bnd[1], -1, tail64(dt.m, tm) ? 1 : 0,
                                  tail_cols(dt.n, tn)});
            continue;
          }
          for (int ch = 0; ch < nc; ++ch)
            t2[g].push_back(DTile{r.task, tm, tn, bnd[ch], bnd[ch + 1], slots[g] + ch, tail64(dt.m, tm) ? 1 : 0,
                                  tail_cols(dt.n, tn)});
          red[g].push_back(DReduce{r.task, tm, tn, slots[g], nc, 0});
          slots[g] += nc;
        }
    }
  }
  // heaviest tiles first within each launch (persistent CTAs take tiles round-robin)
  auto tile_work = [&](const DTile& t, const std::vector<DGemmPair>& pr) {
    int64_t w = 0;
    for (int q = t.p0; q < t.p1; ++q) w += (pr[q].k + kPkTileK - 1) / kPkTileK;
    return w;
  };
  std::vector<DTile> all1, all2;
  std::vector<DReduce> allr;
  for (int g = 0; g < ng; ++g) {
    std::stable_sort(t1[g].begin(), t1[g].end(),
                     [&](const DTile& a, const DTile& b) { return tile_work(a, p.s1.h_pairs) > tile_work(b, p.s1.h_pairs); });
    std::stable_sort(t2[g].begin(), t2[g].end(),
                     [&](const DTile& a, const DTile& b) { return tile_work(a, p.s2.h_pairs) > tile_work(b, p.s2.h_pairs); });
    SigmaPlan::Group G;
    G.t1_begin = static_cast<int>(all1.size());
    G.t1_count = static_cast<int>(t1[g].size());
    G.t2_begin = static_cast<int>(all2.size());
    G.t2_count = static_cast<int>(t2[g].size());
    G.r_begin = static_cast<int>(allr.size());
    G.r_count = static_cast<int>(red[g].size());
    G.nslots = slots[g];
    p.group_slots = std::max(p.group_slots, slots[g]);
    all1.insert(all1.end(), t1[g].begin(), t1[g].end());
    all2.insert(all2.end(), t2[g].begin(), t2[g].end());
    allr.insert(allr.end(), red[g].begin(), red[g].end());
    p.groups.push_back(G);
  }
  p.gt1.upload(all1, ctx.stream);
  p.gt2.upload(all2, ctx.stream);
  p.gred.upload(allr, ctx.stream);
  p.gtasks1.upload(tasks1, ctx.stream);
  p.gpk2.upload(pairs2, ctx.stream);
  p.group_budget = budget;
}

static void sigma_run_pk_whole(Context& ctx, SigmaPlan& p, double* sigma);
static void sigma_groups_run(Context& ctx, SigmaPlan& p, double* sigma);

// sigma += H psi over the w-groups through the plan's CUDA graph (captured on first
// use, and again whenever a buffer it refers to has moved): the graph zeroes the
// staged result and runs every group's launches; one axpy adds it to sigma.
static void sigma_groups_graph(Context& ctx, SigmaPlan& p, double* sigma) {
  const int64_t n = std::max<int64_t>(p.psi_layout.nnz, 1);
  p.staged.ensure(size_t(n) * sizeof(double), ctx.stream);
  p.group_scr.ensure(std::max<int64_t>(p.group_scr_bytes, 16), ctx.stream);
  ctx.gemm_part.ensure(std::max<size_t>(size_t(p.group_slots) * kTcTileM * kTcTileN * sizeof(double), 16),
                       ctx.stream);
  int* err = device_err_flag(ctx);
  const std::vector<const void*> ptrs = {p.pk_L.buf.p, p.pk_R.buf.p, p.pk_psi.buf.p, p.group_scr.p,
                                         ctx.gemm_part.p,  p.staged.p,   err};
  if (!p.graph || ptrs != p.graph_ptrs) {
    p.drop_graph();
    cudaGraph_t g = nullptr;
    cuda_check(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
    cuda_check(cudaMemsetAsync(p.staged.p, 0, size_t(n) * sizeof(double), ctx.stream), "staged zero");
    sigma_groups_run(ctx, p, p.staged.as<double>());
    cuda_check(cudaStreamEndCapture(ctx.stream, &g), "graph capture end");
    cudaError_t e = cudaGraphInstantiate(&p.graph, g, 0);
    cudaGraphDestroy(g);
    cuda_check(e, "graph instantiate");
    p.graph_ptrs = ptrs;
  }
  cuda_check(cudaGraphLaunch(p.graph, ctx.stream), "graph launch");
  launch_axpy(sigma, p.staged.as<double>(), n, 1.0, ctx.stream);
  ctx.kernel_launches += 1;
}

// sigma += H psi over the w-groups of the plan (packed operators and psi in place).
static void sigma_groups_run(Context& ctx, SigmaPlan& p, double* sigma) {
  p.group_scr.ensure(std::max<int64_t>(p.group_scr_bytes, 16), ctx.stream);
  ctx.gemm_part.ensure(std::max<size_t>(size_t(p.group_slots) * kTcTileM * kTcTileN * sizeof(double), 16),
                       ctx.stream);
  double* part = ctx.gemm_part.as<double>();
  int* err = device_err_flag(ctx);
  for (const SigmaPlan::Group& G : p.groups) {
    if (G.t1_count)
      launch_gemm_pk(p.pk_L.buf.as<uint8_t>(), p.pk_psi.buf.as<uint8_t>(), 1.0, nullptr, p.group_scr.as<uint8_t>(),
                     p.gt1.get() + G.t1_begin, G.t1_count, p.gtasks1.get(), p.pk1.get(), nullptr,
                     p.scr1_single ? kOutPackedSingle : kOutPackedSplit, p.stage1_single(), err, ctx.stream,
                     ctx.device_timeout_ns);
    if (G.t2_count)
      launch_gemm_pk(p.group_scr.as<uint8_t>(), p.pk_R.buf.as<uint8_t>(), 1.0, sigma, nullptr,
                     p.gt2.get() + G.t2_begin, G.t2_count, p.s2.dtasks.get(), p.gpk2.get(), part, kOutFP64,
                     p.stage2_single(), err, ctx.stream, ctx.device_timeout_ns);
    if (G.r_count)
      launch_gemm_pk_reduce(p.gred.get() + G.r_begin, G.r_count, p.s2.dtasks.get(), 1.0, part, sigma, ctx.stream);
    ctx.kernel_launches += (G.t1_count > 0) + (G.t2_count > 0) + (G.r_count > 0);
  }
}

// Autotuner of the tensor-core schedule: times one H_eff*psi (psi already packed) into
// a scratch result for a few stage-2 split-K granularities (and, for very large
// intermediates, w blocking) and keeps the fastest.  Runs once per plan; plans are
// kept across bonds and sweeps.
// Switches a plan's L*psi intermediate between hi|lo and FP32 tiles (packed layouts of
// L, R and psi are unchanged, so their packed data stays valid; the intermediate's
// buffer is sized by the caller that runs the plan).
void set_scr1_format(Context& ctx, SigmaPlan& p, const Tensor& L, const Tensor& R, bool single) {
  std::lock_guard<std::mutex> lk(p.pk_mu);
  if (p.scr1_single == single && p.pk_built) return;
  p.scr1_single = single;
  p.pk_built = false;
  build_sigma_pk(ctx, p, L, R, p.psi_layout);
  // w groups place the intermediate's blocks by their packed size: rebuild them
  if (!p.groups.empty()) build_sigma_groups(ctx, p, p.group_budget);
  p.drop_graph();
}

static void tune_sigma_groups(Context& ctx, SigmaPlan& p, const Tensor& L, const Tensor& R) {
  const int64_t n = std::max<int64_t>(p.psi_layout.nnz, 1);
  DevBuf out;
  out.ensure(size_t(n) * sizeof(double), ctx.stream);
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "tune event");
  cuda_check(cudaEventCreate(&e1), "tune event");
  const int64_t mb = int64_t(1) << 20;
  // candidates: (w budget, stage-2 CTA target, intermediate format); budget 0 = all of
  // w at once.  w blocking pays per-group pipeline fill and tail costs (measured 2x
  // slower than one pass when the intermediate fits), so it is tried only when the
  // whole-w intermediate is large enough to matter for memory.  The FP32 intermediate
  // halves its HBM bytes but adds shared-memory traffic (the on-chip split), which
  // bounds the kernel on the measured workloads; both are timed.
  struct Cand {
    int64_t budget;
    int target;
    bool single;
  };
  std::vector<Cand> cands;
  for (bool single : {false, true})
    for (int target : {152 * 4, 152 * 8, 152 * 16}) cands.push_back({0, target, single});
  if (p.pk_scr1.bytes > kGroupIntermediateBytes) cands.push_back({128 * mb, 152 * 8, false});
  Cand best = cands[0];
  float best_ms = 0.0f;
  ctx.last_tuning.clear();
  for (const Cand& cand : cands) {
    const int64_t b = cand.budget;
    set_scr1_format(ctx, p, L, R, cand.single);
    p.pk_scr1.buf.ensure(std::max<int64_t>(p.pk_scr1.bytes, 16), ctx.stream);
    if (b > 0) {
      build_sigma_groups(ctx, p, b);
      p.drop_graph();
      if (p.groups.size() < 2) continue;  // no blocking at this budget
    } else {
      tile_tc(p.s2, cand.target);
      p.s2.tiles_tc.upload(p.s2.h_tiles_tc, ctx.stream);
      p.s2.reduce_tc.upload(p.s2.h_reduce_tc, ctx.stream);
    }
    float ms = 0.0f;
    for (int rep = 0; rep < 2; ++rep) {
      cuda_check(cudaMemsetAsync(out.p, 0, size_t(n) * sizeof(double), ctx.stream), "tune zero");
      cuda_check(cudaEventRecord(e0, ctx.stream), "tune record");
      if (b > 0)
        sigma_groups_graph(ctx, p, out.as<double>());
      else
        sigma_run_pk_whole(ctx, p, out.as<double>());
      cuda_check(cudaEventRecord(e1, ctx.stream), "tune record");
      cuda_check(cudaEventSynchronize(e1), "tune sync");
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "tune time");
    }
    ctx.last_tuning.push_back(double(b));
    ctx.last_tuning.push_back(double(cand.target));
    ctx.last_tuning.push_back(cand.single ? 1.0 : 0.0);
    ctx.last_tuning.push_back(ms);
    if (best_ms == 0.0f || ms < best_ms) {
      best = cand;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  set_scr1_format(ctx, p, L, R, best.single);
  p.pk_scr1.buf.ensure(std::max<int64_t>(p.pk_scr1.bytes, 16), ctx.stream);
  p.drop_graph();
  if (best.budget > 0) {
    build_sigma_groups(ctx, p, best.budget);
    p.pk_scr1.buf.release();
  } else {
    p.groups.clear();
    tile_tc(p.s2, best.target);
    p.s2.tiles_tc.upload(p.s2.h_tiles_tc, ctx.stream);
    p.s2.reduce_tc.upload(p.s2.h_reduce_tc, ctx.stream);
  }
  p.group_budget = best.budget;
  p.tuned_ms = best_ms;
}

static void sigma_run_pk(Context& ctx, SigmaPlan& p, const DTensor& L, const DTensor& R, const double* psi,
                         double* sigma) {
  {
    PhaseTimer tm(ctx, kPhSigmaPlan);
    if (!p.pk_built) build_sigma_pk(ctx, p, L, R, p.psi_layout);
    // packed buffers are handed back between bonds; the plan itself is kept
    for (Packed* P : {&p.pk_L, &p.pk_R, &p.pk_psi})
      P->buf.ensure(std::max<int64_t>(P->bytes, 16), ctx.stream);
    // the whole-w intermediate is only needed when w is not blocked (or while tuning)
    if (p.group_budget <= 0) p.pk_scr1.buf.ensure(std::max<int64_t>(p.pk_scr1.bytes, 16), ctx.stream);
    // operators are packed once per (layout, data version)
    if (p.pk_L.src_layout != L.layout_id || p.pk_L.src_version != L.data_version) pack_into(ctx, p.pk_L, L);
    if (p.pk_R.src_layout != R.layout_id || p.pk_R.src_version != R.data_version) pack_into(ctx, p.pk_R, R);
    tm.stop();
    ctx.timers[kPhSigma] -= tm.dt;  // counted as planning, not as H_eff * psi
  }
  launch_pack(p.pk_psi.packs.get(), static_cast<int>(p.pk_psi.h_packs.size()), psi, p.pk_psi.buf.as<uint8_t>(),
              ctx.stream);
  if (p.group_budget < 0) {
    if (ctx.sigma_w_budget < 0) {
      tune_sigma_groups(ctx, p, L, R);
    } else if (ctx.sigma_w_budget > 0) {
      set_scr1_format(ctx, p, L, R, ctx.sigma_fp32_intermediate);
      build_sigma_groups(ctx, p, ctx.sigma_w_budget);
      if (p.groups.size() < 2) {  // the budget does not split w: one pass
        p.groups.clear();
        p.group_budget = 0;
      } else {
        p.group_budget = ctx.sigma_w_budget;
        p.pk_scr1.buf.release();
      }
    } else {
      set_scr1_format(ctx, p, L, R, ctx.sigma_fp32_intermediate);
      p.pk_scr1.buf.ensure(std::max<int64_t>(p.pk_scr1.bytes, 16), ctx.stream);
      if (ctx.sigma_target_tiles > 0) {
        tile_tc(p.s2, ctx.sigma_target_tiles);
        p.s2.tiles_tc.upload(p.s2.h_tiles_tc, ctx.stream);
        p.s2.reduce_tc.upload(p.s2.h_reduce_tc, ctx.stream);
      }
      p.group_budget = 0;
    }
  }
  if (p.group_budget > 0) {
    sigma_groups_graph(ctx, p, sigma);
    ctx.kernel_launches += 1;
    return;
  }
  sigma_run_pk_whole(ctx, p, sigma);
}

// Both stages over all of w at once (the packed L*psi intermediate in HBM).
static void sigma_run_pk_whole(Context& ctx, SigmaPlan& p, double* sigma) {
  int* err = device_err_flag(ctx);
  if (p.stack1)
    launch_gemm_pk(p.pk_L.buf.as<uint8_t>(), p.pk_psi.buf.as<uint8_t>(), 1.0, nullptr, p.pk_scr1.buf.as<uint8_t>(),
                   p.st1.get(), static_cast<int>(p.h_st1.size()), p.pk_tasks1.get(), p.stpk1.get(), nullptr,
                   p.scr1_single ? kOutPackedSingle : kOutPackedSplit, p.stage1_single(), err, ctx.stream,
                   ctx.device_timeout_ns, p.row_map.get());
  else
    launch_gemm_pk(p.pk_L.buf.as<uint8_t>(), p.pk_psi.buf.as<uint8_t>(), 1.0, nullptr, p.pk_scr1.buf.as<uint8_t>(),
                   p.s1.tiles_tc.get(), static_cast<int>(p.s1.h_tiles_tc.size()), p.pk_tasks1.get(), p.pk1.get(),
                   nullptr, p.scr1_single ? kOutPackedSingle : kOutPackedSplit, p.stage1_single(), err, ctx.stream,
                   ctx.device_timeout_ns);
  ctx.gemm_part.ensure(std::max<size_t>(p.s2.partial_bytes_tc(), 16), ctx.stream);
  double* part = ctx.gemm_part.as<double>();
  launch_gemm_pk(p.pk_scr1.buf.as<uint8_t>(), p.pk_R.buf.as<uint8_t>(), 1.0, sigma, nullptr,
                 p.s2.tiles_tc.get(), static_cast<int>(p.s2.h_tiles_tc.size()), p.s2.dtasks.get(), p.pk2.get(), part,
                 kOutFP64, p.stage2_single(), err, ctx.stream, ctx.device_timeout_ns);
  if (p.s2.nslots_tc > 0)
    launch_gemm_pk_reduce(p.s2.reduce_tc.get(), static_cast<int>(p.s2.h_reduce_tc.size()), p.s2.dtasks.get(), 1.0,
                          part, sigma, ctx.stream);
  ctx.kernel_launches += 3 + (p.s2.nslots_tc > 0);
}

static void sigma_run(Context& ctx, SigmaPlan& p, const DTensor& L, const DTensor& R, const double* psi,
                      double* sigma, int precision) {
  if (precision != kFP64) {
    sigma_run_pk(ctx, p, L, R, psi, sigma);
  } else {
    ctx.scr1.ensure(std::max<int64_t>(p.scr1.nnz, 1) * sizeof(double), ctx.stream);
    double* scr = ctx.scr1.as<double>();
    if (p.scr1.nnz) cuda_check(cudaMemsetAsync(scr, 0, p.scr1.nnz * sizeof(double), ctx.stream), "scr1 zero");
    ctx.gemm_part.ensure(std::max(p.s1.partial_bytes(), p.s2.partial_bytes()), ctx.stream);
    double* part = ctx.gemm_part.as<double>();
    p.s1.run(1.0, L.d, psi, scr, part, ctx.stream);
    p.s2.run(1.0, scr, R.d, sigma, part, ctx.stream);
    ctx.kernel_launches += 2 + (p.s1.nslots > 0) + (p.s2.nslots > 0);
  }
  ctx.sigma_flops += p.flops;
  ctx.sigma_calls += 1;
}

std::vector<double> sigma_plan_stats(Context& ctx, const Tensor& L, const Tensor& R, const Tensor& psi) {
  SigmaPlan& p = sigma_plan(ctx, L, R, psi);
  ensure_sigma_pk(ctx, p, L, R);
  auto work = [&](const std::vector<DTile>& tiles, const std::vector<DPkPair>& pairs, double* slices) {
    double s = 0.0, w = 0.0;
    for (const DTile& t : tiles) {
      // one K slice of the tile (64-row tails counted at their size)
      const double tf = 2.0 * (t.h64 ? 64 : kTcTileM) * t.nt * kPkTileK;
      for (int q = t.p0; q < t.p1; ++q) {
        s += pairs[q].nks;
        w += pairs[q].nks * tf;
      }
    }
    *slices = s;
    return w;
  };
  double sl1 = 0.0, sl2 = 0.0;
  const std::vector<DTile>& t1 = p.stack1 ? p.h_st1 : p.s1.h_tiles_tc;
  const double w1 = work(t1, p.stack1 ? p.h_stpk1 : p.h_pk1, &sl1);
  const double w2 = work(p.s2.h_tiles_tc, p.h_pk2, &sl2);
  // FLOPs with one dimension padded at a time (rows to 128, columns to 64, K to 32)
  auto padded = [](const GemmPlan& g, double* pm, double* pn, double* pk) {
    auto up = [](int x, int q) { return double((x + q - 1) / q * q); };
    for (const DGemmTask& t : g.h_tasks)
      for (int q = t.p0; q < t.p1; ++q) {
        const double m = t.m, n = t.n, k = g.h_pairs[q].k;
        *pm += 2.0 * up(t.m, kTcTileM) * n * k;
        *pn += 2.0 * m * up(t.n, kTcTileN) * k;
        *pk += 2.0 * m * n * up(g.h_pairs[q].k, kPkTileK);
      }
  };
  double pm1 = 0, pn1 = 0, pk1 = 0, pm2 = 0, pn2 = 0, pk2 = 0;
  padded(p.s1, &pm1, &pn1, &pk1);
  padded(p.s2, &pm2, &pn2, &pk2);
  auto tails = [](const std::vector<DTile>& tiles, bool rows) {
    double c = 0.0;
    for (const DTile& t : tiles) c += rows ? t.h64 : (t.nt < kTcTileN ? 1 : 0);
    return c;
  };
  // tile FLOPs if a block's last row tile were 64 rows high where its remainder fits
  auto tile64 = [](const GemmPlan& g) {
    double s = 0.0;
    for (const DGemmTask& t : g.h_tasks) {
      const int full = t.m / kTcTileM, rem = t.m % kTcTileM;
      const double rows = double(full) * kTcTileM + (rem == 0 ? 0 : rem <= 64 ? 64 : kTcTileM);
      const double cols = double((t.n + kTcTileN - 1) / kTcTileN * kTcTileN);
      for (int q = t.p0; q < t.p1; ++q) s += 2.0 * rows * cols * ((g.h_pairs[q].k + kPkTileK - 1) / kPkTileK * kPkTileK);
    }
    return s;
  };
  return {p.s1.flops,
          p.s2.flops,
          w1,
          w2,
          sl1,
          sl2,
          double(t1.size()),
          double(p.s2.h_tiles_tc.size()),
          double(p.pk_L.bytes),
          double(p.pk_R.bytes),
          double(p.pk_scr1.bytes),
          double(p.pk_psi.bytes),
          double(p.scr1.nnz),
          pm1,
          pn1,
          pk1,
          pm2,
          pn2,
          pk2,
          tile64(p.s1),
          tile64(p.s2),
          tails(t1, true) + tails(p.s2.h_tiles_tc, true),
          tails(t1, false) + tails(p.s2.h_tiles_tc, false)};
}

void ensure_sigma_pk(Context& ctx, SigmaPlan& p, const Tensor& L, const Tensor& R) {
  std::lock_guard<std::mutex> lk(p.pk_mu);
  if (!p.pk_built) build_sigma_pk(ctx, p, L, R, p.psi_layout);
}

void apply_sigma(Context& ctx, SigmaPlan& p, const DTensor& L, const DTensor& R, const double* psi, double* sigma,
                 int precision) {
  sigma_run(ctx, p, L, R, psi, sigma, precision);
}

// Device error flag of the tensor-core kernels (zeroed on first use).
int* device_err_flag(Context& ctx) {
  if (!ctx.err_flag.p) {
    ctx.err_flag.ensure(sizeof(int), ctx.stream);
    cuda_check(cudaMemsetAsync(ctx.err_flag.p, 0, sizeof(int), ctx.stream), "err flag zero");
  }
  return ctx.err_flag.as<int>();
}

// Throws DEVICE_TIMEOUT when a tensor-core kernel gave up waiting for its MMAs.
void check_device_error(Context& ctx) {
  if (!ctx.err_flag.p) return;
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, ctx.err_flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream), "err d2h");
  ctx.sync();
  if (h) {
    cuda_check(cudaMemsetAsync(ctx.err_flag.p, 0, sizeof(int), ctx.stream), "err flag reset");
    throw Error(kDeviceTimeout, "tensor-core kernel: MMA completion wait timed out");
  }
}

void compute_sigma_vector(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& psi, DTensor& sigma) {
  if (sigma.nnz != psi.nnz || sigma.tags != psi.tags)
    throw Error(kInvalidArgument, "compute_sigma_vector: sigma must have the wavefunction's block layout");
  SigmaPlan& p = sigma_plan(ctx, L, R, psi);
  sigma_run(ctx, p, L, R, psi.d, sigma.d, ctx.precision);
}

double sigma_device_time(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& psi, DTensor& sigma,
                         int reps) {
  SigmaPlan& p = sigma_plan(ctx, L, R, psi);
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event create");
  cuda_check(cudaEventCreate(&e1), "event create");
  cuda_check(cudaEventRecord(e0, ctx.stream), "event record");
  for (int r = 0; r < reps; ++r) sigma_run(ctx, p, L, R, psi.d, sigma.d, ctx.precision);
  cuda_check(cudaEventRecord(e1, ctx.stream), "event record");
  cuda_check(cudaEventSynchronize(e1), "event sync");
  float ms = 0.f;
  cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event time");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return double(ms) / 1e3 / reps;
}

// ---------------------------------------------------------------------------
// diagonal
// ---------------------------------------------------------------------------
DiagPlan& diag_plan(Context& ctx, const Tensor& L, const Tensor& R, const Tensor& diag) {
  auto key = std::make_tuple(L.layout_id, R.layout_id, diag.layout_id);
  if (DiagPlan* hit = find_plan(ctx, ctx.diag_plans, key)) return *hit;
  PhaseTimer tm(ctx, kPhSigmaPlan);
  auto p = std::make_unique<DiagPlan>();
  // tied arrays: row sector -> [(w, block slot)] for blocks (i, w, i), ascending w
  auto tied = [](const Tensor& t) {
    std::map<int, std::vector<std::pair<int, int32_t>>> m;
    int idx[kMaxRank];
    for (size_t b = 0; b < t.tags.size(); ++b) {
      t.sh.index(t.tags[b], idx);
      if (idx[0] == idx[2]) m[idx[0]].push_back({idx[1], static_cast<int32_t>(b)});
    }
    for (auto& kv : m) std::sort(kv.second.begin(), kv.second.end());
    return m;
  };
  auto lt = tied(L);
  auto rt = tied(R);
  int idx[kMaxRank];
  for (size_t b = 0; b < diag.tags.size(); ++b) {
    diag.sh.index(diag.tags[b], idx);
    auto li = lt.find(idx[0]);
    auto ri = rt.find(idx[1]);
    if (li == lt.end() || ri == rt.end()) continue;
    DDiagTask t;
    t.out_off = diag.offsets[b];
    t.m = diag.sh.dshape[0][idx[0]];
    t.n = diag.sh.dshape[1][idx[1]];
    t.p0 = static_cast<int>(p->h_pairs.size());
    std::vector<std::pair<int64_t, int64_t>> refp;
    size_t x = 0, y = 0;
    const auto& lv = li->second;
    const auto& rv = ri->second;
    while (x < lv.size() && y < rv.size()) {
      if (lv[x].first == rv[y].first) {
        p->h_pairs.push_back(DDiagPair{L.offsets[lv[x].second], R.offsets[rv[y].second]});
        refp.push_back({L.tags[lv[x].second], R.tags[rv[y].second]});
        ++x;
        ++y;
      } else if (lv[x].first < rv[y].first) {
        ++x;
      } else {
        ++y;
      }
    }
    t.p1 = static_cast<int>(p->h_pairs.size());
    if (t.p1 == t.p0) continue;
    p->h_tasks.push_back(t);
    p->ref.push_back({diag.tags[b], std::move(refp)});
  }
  for (const DDiagTask& t : p->h_tasks)
    p->max_tiles = std::max(p->max_tiles, ((t.m + 31) / 32) * ((t.n + 31) / 32));
  p->tasks.upload(p->h_tasks, ctx.stream);
  p->pairs.upload(p->h_pairs, ctx.stream);
  return insert_plan(ctx, ctx.diag_plans, key, std::move(p));
}

void compute_diagonal_elements(Context& ctx, const DTensor& L, const DTensor& R, DTensor& diag) {
  DiagPlan& p = diag_plan(ctx, L, R, diag);
  launch_diag(p.tasks.get(), static_cast<int>(p.h_tasks.size()), p.pairs.get(), L.d, R.d, diag.d, p.max_tiles,
              ctx.stream);
  ctx.kernel_launches += 1;
}

// ---------------------------------------------------------------------------
// renormalize (merged operator)
// ---------------------------------------------------------------------------
static std::unique_ptr<RenormPlan> build_renorm_plan(Context& ctx, bool forward, const Tensor& opr0,
                                                     const Tensor& bra, const Tensor& ket) {
  auto rp = std::make_unique<RenormPlan>();
  Tensor cbra = conj_view(bra);
  int K1 = 0, K2 = 0;
  Shape s2;
  if (forward) {
    Shape s1 = gemm_result_shape(kTrans, kNoTrans, cbra.sh, opr0.sh, 3, &K1);
    auto t1 = enumerate_gemm(kTrans, kNoTrans, cbra, opr0, s1, K1);
    layout_from_tasks(rp->scr, s1, t1);
    build_gemm_plan(rp->p1, kTrans, kNoTrans, cbra, opr0, rp->scr, K1, std::move(t1));
    s2 = gemm_result_shape(kNoTrans, kNoTrans, rp->scr.sh, ket.sh, 3, &K2);
  } else {
    Shape s1 = gemm_result_shape(kNoTrans, kNoTrans, cbra.sh, opr0.sh, 3, &K1);
    auto t1 = enumerate_gemm(kNoTrans, kNoTrans, cbra, opr0, s1, K1);
    layout_from_tasks(rp->scr, s1, t1);
    build_gemm_plan(rp->p1, kNoTrans, kNoTrans, cbra, opr0, rp->scr, K1, std::move(t1));
    s2 = gemm_result_shape(kNoTrans, kTrans, rp->scr.sh, ket.sh, 3, &K2);
  }
  const Trans tb2 = forward ? kNoTrans : kTrans;
  auto t2 = enumerate_gemm(kNoTrans, tb2, rp->scr, ket, s2, K2);
  layout_from_tasks(rp->out, s2, t2);
  build_gemm_plan(rp->p2, kNoTrans, tb2, rp->scr, ket, rp->out, K2, std::move(t2));
  rp->p1.upload(ctx.stream);
  rp->p2.upload(ctx.stream);
  return rp;
}

RenormPlan& renorm_plan(Context& ctx, bool forward, const Tensor& opr0, const Tensor& bra, const Tensor& ket) {
  const auto key = std::make_tuple(forward ? 1 : 0, opr0.layout_id, bra.layout_id, ket.layout_id);
  if (RenormPlan* hit = find_plan(ctx, ctx.renorm_plans, key)) return *hit;
  return insert_plan(ctx, ctx.renorm_plans, key, build_renorm_plan(ctx, forward, opr0, bra, ket));
}

std::unique_ptr<DTensor> renormalize(Context& ctx, bool forward, const DTensor& opr0, const DTensor& bra,
                                     const DTensor& ket) {
  PhaseTimer tplan(ctx, kPhRenormPlan);
  RenormPlan& rp = renorm_plan(ctx, forward, opr0, bra, ket);
  const bool split = ctx.precision == kSplitTF32All;
  if (split && !rp.split_built) {
    build_split_gemm(ctx, rp.g1, rp.p1, conj_view(bra), opr0);
    build_split_gemm(ctx, rp.g2, rp.p2, rp.scr, ket);
    rp.split_built = true;
  }
  auto out = std::make_unique<DTensor>();
  static_cast<Tensor&>(*out) = rp.out;
  tplan.stop();
  PhaseTimer trun(ctx, kPhRenormRun);
  out->ctx = &ctx;
  out->alloc_device(ctx.stream, true);
  const int64_t scr_nnz = rp.scr.nnz;
  ctx.scr2.ensure(std::max<int64_t>(scr_nnz, 1) * sizeof(double), ctx.stream);
  double* sp = ctx.scr2.as<double>();
  if (scr_nnz) cuda_check(cudaMemsetAsync(sp, 0, scr_nnz * sizeof(double), ctx.stream), "renorm scr zero");
  if (split) {
    run_split_gemm(ctx, rp.g1, rp.p1, 1.0, bra.d, opr0.d, sp);
    run_split_gemm(ctx, rp.g2, rp.p2, 1.0, sp, ket.d, out->d);
    for (Packed* P : {&rp.g1.pa, &rp.g1.pb, &rp.g2.pa, &rp.g2.pb}) P->buf.release();
    check_device_error(ctx);
  } else {
    ctx.gemm_part.ensure(std::max(rp.p1.partial_bytes(), rp.p2.partial_bytes()), ctx.stream);
    rp.p1.run(1.0, bra.d, opr0.d, sp, ctx.gemm_part.as<double>(), ctx.stream);
    rp.p2.run(1.0, sp, ket.d, out->d, ctx.gemm_part.as<double>(), ctx.stream);
    ctx.kernel_launches += 2;
  }
  return out;
}

// ---------------------------------------------------------------------------
// merged super-block operators (scatter of scalar MPO blocks)
// ---------------------------------------------------------------------------
static std::unique_ptr<MergePlan> build_merge_plan(Context& ctx, bool forward, const DTensor& mpo,
                                                   const Tensor& opr) {
  for (size_t b = 0; b < mpo.tags.size(); ++b)
    if ((b + 1 < mpo.tags.size() ? mpo.offsets[b + 1] : mpo.nnz) - mpo.offsets[b] != 1)
      throw Error(kInvalidArgument, "merged operator: MPO blocks must be scalars (1x1x1x1)");
  // Forward:  mL[A=(a,s), v, A'=(x,t)] = sum_w W[w,s,t,v] L[a,w,x]
  // Backward: mR[B=(s,b), w, B'=(t,y)] = sum_v W[w,s,t,v] R[b,v,y]
  // Every environment block (a,c,x) (c = w forward, v backward) meets the MPO
  // entries that share c; a destination sub-block is fixed by the environment's
  // outer pair (a,x) and the entry's column (s,t,u) (u = v forward, w backward).
  // The plan is built group by group over (a,x) with a dense column stamp, so its
  // cost is linear in the number of contributions (no sorting, no hashing).
  const int ns = mpo.sh.nsec(1), nt = mpo.sh.nsec(2);
  const int c_axis = forward ? 0 : 3, u_axis = forward ? 3 : 0;
  const int nu = mpo.sh.nsec(u_axis);
  MergeInfo mb, mk;
  auto out = std::make_unique<DTensor>();
  out->sh.rank = 3;
  out->sh.q = opr.sh.q + mpo.sh.q;
  if (forward) {
    mb = MergeInfo({opr.sh.qshape[0], mpo.sh.qshape[1]}, {opr.sh.dshape[0], mpo.sh.dshape[1]});
    mk = MergeInfo({opr.sh.qshape[2], mpo.sh.qshape[2]}, {opr.sh.dshape[2], mpo.sh.dshape[2]});
  } else {
    mb = MergeInfo({mpo.sh.qshape[1], opr.sh.qshape[0]}, {mpo.sh.dshape[1], opr.sh.dshape[0]});
    mk = MergeInfo({mpo.sh.qshape[2], opr.sh.qshape[2]}, {mpo.sh.dshape[2], opr.sh.dshape[2]});
  }
  out->sh.qshape = {mb.q_merged, mpo.sh.qshape[u_axis], mk.q_merged};
  out->sh.dshape = {mb.d_merged, mpo.sh.dshape[u_axis], mk.d_merged};
  out->sh.finalize();
  // MPO entries by contracted index c, in block order: column id (s*nt + t)*nu + u
  const int nc = mpo.sh.nsec(c_axis);
  std::vector<int32_t> row_ptr(nc + 1, 0), ent_col, ent_st;
  std::vector<double> ent_coef;
  {
    std::vector<std::array<int, 4>> mi(mpo.tags.size());
    for (size_t b = 0; b < mpo.tags.size(); ++b) {
      mpo.sh.index(mpo.tags[b], mi[b].data());
      row_ptr[mi[b][c_axis] + 1]++;
    }
    for (int c = 0; c < nc; ++c) row_ptr[c + 1] += row_ptr[c];
    ent_col.resize(mpo.tags.size());
    ent_coef.resize(mpo.tags.size());
    ent_st.resize(mpo.tags.size());
    std::vector<int32_t> fill(row_ptr.begin(), row_ptr.end() - 1);
    for (size_t b = 0; b < mpo.tags.size(); ++b) {
      const int e = fill[mi[b][c_axis]]++;
      ent_col[e] = (mi[b][1] * nt + mi[b][2]) * nu + mi[b][u_axis];
      ent_coef[e] = mpo.host[mpo.offsets[b]];
      ent_st[e] = static_cast<int32_t>(b);  // MPO block slot of the entry
    }
  }
  // environment blocks grouped by outer pair (a,x), contracted index ascending
  const int nx = opr.sh.nsec(2);
  std::vector<std::array<int, 3>> oi(opr.tags.size());
  std::vector<int32_t> order(opr.tags.size());
  for (size_t b = 0; b < opr.tags.size(); ++b) {
    opr.sh.index(opr.tags[b], oi[b].data());
    order[b] = static_cast<int32_t>(b);
  }
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
    return int64_t(oi[x][0]) * nx + oi[x][2] < int64_t(oi[y][0]) * nx + oi[y][2];
  });
  // pass 1: destinations of every group, with their contribution counts
  struct Dst {
    int32_t col, cnt;
    int64_t otag;
  };
  std::vector<Dst> dsts;
  std::vector<int64_t> group_first;  // [g] -> first destination of group g
  std::vector<int32_t> group_src;    // [g] -> first entry of order[] in group g
  const int ncols_all = ns * nt * nu;
  std::vector<int32_t> stamp(ncols_all, -1), where(ncols_all, 0);
  const int64_t nsparse = out->sh.nsparse;
  std::vector<uint64_t> present((nsparse + 63) / 64, 0);
  for (size_t o = 0; o < order.size();) {
    const int a = oi[order[o]][0], x = oi[order[o]][2];
    size_t o1 = o;
    while (o1 < order.size() && oi[order[o1]][0] == a && oi[order[o1]][2] == x) ++o1;
    const int g = static_cast<int>(group_first.size());
    group_first.push_back(static_cast<int64_t>(dsts.size()));
    group_src.push_back(static_cast<int32_t>(o));
    for (size_t q = o; q < o1; ++q) {
      const int c = oi[order[q]][1];
      for (int e = row_ptr[c]; e < row_ptr[c + 1]; ++e) {
        const int col = ent_col[e];
        if (stamp[col] != g) {
          stamp[col] = g;
          where[col] = static_cast<int32_t>(dsts.size());
          const int u = col % nu, st = col / nu, sidx = st / nt, tidx = st % nt;
          const int ipr = forward ? a * ns + sidx : sidx * opr.sh.nsec(0) + a;
          const int ipc = forward ? x * nt + tidx : tidx * nx + x;
          int ti[3] = {mb.merged_of[ipr], u, mk.merged_of[ipc]};
          if (!out->sh.allowed(ti)) throw Error(kQShapeMismatch, "merged operator: contribution not allowed");
          const int64_t otag = out->sh.tag(ti);
          present[otag >> 6] |= uint64_t(1) << (otag & 63);
          dsts.push_back(Dst{col, 0, otag});
        }
        dsts[where[col]].cnt++;
      }
    }
    o = o1;
  }
  group_first.push_back(static_cast<int64_t>(dsts.size()));
  group_src.push_back(static_cast<int32_t>(order.size()));
  // output blocks: the marked tags in ascending order; slot of a tag by rank
  std::vector<int64_t> tags;
  std::vector<int32_t> rank_before(present.size() + 1, 0);
  for (size_t w = 0; w < present.size(); ++w) {
    rank_before[w + 1] = rank_before[w] + __builtin_popcountll(present[w]);
    for (uint64_t bits = present[w]; bits; bits &= bits - 1)
      tags.push_back(int64_t(w) * 64 + __builtin_ctzll(bits));
  }
  out->set_blocks(tags);
  auto slot_of = [&](int64_t t) {
    return rank_before[t >> 6] + __builtin_popcountll(present[t >> 6] & ((uint64_t(1) << (t & 63)) - 1));
  };
  // pass 2: destination records and their sources (ascending contracted index)
  std::vector<DScatterDst> hd;
  std::vector<DScatterSrc> hs;
  hd.reserve(dsts.size());
  {
    int64_t total = 0;
    for (const Dst& d : dsts) total += d.cnt;
    hs.resize(total);
  }
  std::vector<int32_t> fill(ncols_all, 0);
  int64_t next_src = 0;
  for (size_t g = 0; g + 1 < group_first.size(); ++g) {
    for (int64_t di = group_first[g]; di < group_first[g + 1]; ++di) {
      const Dst& d = dsts[di];
      fill[d.col] = static_cast<int32_t>(next_src);
      const int st = d.col / nu, sidx = st / nt, tidx = st % nt;
      const int32_t first = group_src[g];
      const int a = oi[order[first]][0], x = oi[order[first]][2];
      const int da = opr.sh.dshape[0][a], dx = opr.sh.dshape[2][x];
      const int ipr = forward ? a * ns + sidx : sidx * opr.sh.nsec(0) + a;
      const int ipc = forward ? x * nt + tidx : tidx * nx + x;
      int ti[3];
      out->sh.index(d.otag, ti);
      const int dcols = out->sh.dshape[2][ti[2]];
      DScatterDst r;
      r.dst_off = out->offsets[slot_of(d.otag)] + int64_t(mb.offset_packed[ipr]) * dcols + mk.offset_packed[ipc];
      r.rows = da * mpo.sh.dshape[1][sidx];
      r.cols = dx * mpo.sh.dshape[2][tidx];
      r.dld = dcols;
      r.s0 = static_cast<int>(next_src);
      r.s1 = static_cast<int>(next_src + d.cnt);
      r.pad = slot_of(d.otag);
      next_src += d.cnt;
      if (r.rows > 0 && r.cols > 0) hd.push_back(r);
    }
    for (int32_t q = group_src[g]; q < group_src[g + 1]; ++q) {
      const int32_t ob = order[q];
      const int c = oi[ob][1];
      const int sld = opr.sh.dshape[2][oi[ob][2]];
      for (int e = row_ptr[c]; e < row_ptr[c + 1]; ++e)
        hs[fill[ent_col[e]]++] = DScatterSrc{opr.offsets[ob], sld, ent_st[e], ent_coef[e]};
    }
  }
  auto plan = std::make_unique<MergePlan>();
  plan->layout = static_cast<const Tensor&>(*out);
  plan->dst.upload(hd, ctx.stream);
  plan->src.upload(hs, ctx.stream);
  plan->ndst = static_cast<int>(hd.size());
  plan->h_dst = std::move(hd);
  plan->src_entry.resize(hs.size());
  for (size_t i = 0; i < hs.size(); ++i) plan->src_entry[i] = hs[i].pad;
  plan->nentries = static_cast<int>(mpo.tags.size());
  return plan;
}

static MergePlan& merge_plan_mut(Context& ctx, bool forward, const DTensor& mpo, const Tensor& opr) {
  const auto key = std::make_tuple(forward ? 1 : 0, mpo.layout_id, mpo.data_version, opr.layout_id);
  if (MergePlan* hit = find_plan(ctx, ctx.merge_plans, key)) return *hit;
  return insert_plan(ctx, ctx.merge_plans, key, build_merge_plan(ctx, forward, mpo, opr));
}

const MergePlan& merge_plan(Context& ctx, bool forward, const DTensor& mpo, const Tensor& opr) {
  return merge_plan_mut(ctx, forward, mpo, opr);
}

// dE/dW[e] = sum over the scatter records of MPO block e of <Y_sub, env_block>,
// with Y = dE/d(merged operator) laid out as any tensor whose blocks carry the
// merged operator's sector indices (the adjoint of compute_merged_operator).
std::vector<double> mpo_gradient(Context& ctx, bool forward, const DTensor& mpo, const DTensor& opr,
                                 const DTensor& Y) {
  MergePlan& plan = merge_plan_mut(ctx, forward, mpo, opr);
  if (Y.sh.rank != 3) throw Error(kInvalidArgument, "mpo gradient: adjoint operator must have 3 indices");
  for (int i = 0; i < 3; ++i)
    if (Y.sh.dshape[i] != plan.layout.sh.dshape[i])
      throw Error(kInvalidArgument, "mpo gradient: adjoint operator sectors differ from the merged operator's");
  if (!plan.adj_built) {
    std::vector<int> ptr(plan.nentries + 1, 0), idx(plan.src_entry.size());
    for (int32_t e : plan.src_entry) ptr[e + 1]++;
    for (int e = 0; e < plan.nentries; ++e) ptr[e + 1] += ptr[e];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (size_t s = 0; s < plan.src_entry.size(); ++s) idx[fill[plan.src_entry[s]]++] = static_cast<int>(s);
    plan.adj_ptr.upload(ptr, ctx.stream);
    plan.adj_idx.upload(idx, ctx.stream);
    plan.adj_built = true;
  }
  // destinations rebased onto Y's blocks (absent blocks: Y = 0 there)
  std::vector<DScatterDst> yd(plan.h_dst);
  for (DScatterDst& d : yd) {
    const int64_t tag = plan.layout.tags[d.pad];
    const int32_t ys = Y.find(tag);
    d.dst_off = ys < 0 ? -1 : Y.offsets[ys] + (d.dst_off - plan.layout.offsets[d.pad]);
  }
  DevArray<DScatterDst> dyd;
  dyd.upload(yd, ctx.stream);
  DevBuf g, G;
  g.ensure(std::max<size_t>(plan.src_entry.size(), 1) * sizeof(double), ctx.stream);
  G.ensure(std::max(plan.nentries, 1) * sizeof(double), ctx.stream);
  cuda_check(cudaMemsetAsync(g.p, 0, std::max<size_t>(plan.src_entry.size(), 1) * sizeof(double), ctx.stream),
             "gradient zero");
  launch_adjoint_scatter(dyd.get(), static_cast<int>(yd.size()), plan.src.get(), Y.d, opr.d, g.as<double>(),
                         ctx.stream);
  launch_segment_sum(plan.adj_ptr.get(), plan.adj_idx.get(), g.as<double>(), plan.nentries, G.as<double>(),
                     ctx.stream);
  ctx.kernel_launches += 2;
  std::vector<double> out(plan.nentries);
  if (plan.nentries)
    cuda_check(cudaMemcpyAsync(out.data(), G.p, plan.nentries * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream),
               "gradient d2h");
  ctx.sync();
  return out;
}

// Gradient of E = <psi| H_eff |psi> (psi normalised, merged two-site form) with
// respect to the scalar blocks of both site MPOs of the bond.
void bond_mpo_gradient(Context& ctx, const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr,
                       const DTensor& ropr, const DTensor& psi, std::vector<double>& gl, std::vector<double>& gr) {
  auto mL = compute_merged_operator(ctx, true, lmpo, lopr);
  auto mR = compute_merged_operator(ctx, false, rmpo, ropr);
  // dE/dmL[A,w,A'] = sum psi[A,B] mR[B,w,B'] psi[A',B'] (a backward renormalisation
  // with psi as bra and ket); dE/dmR likewise forward.  These contractions follow
  // the context's precision (split when H_eff * psi is split).
  const int saved = ctx.precision;
  if (ctx.precision != kFP64) ctx.precision = kSplitTF32All;
  std::unique_ptr<DTensor> Y, Z;
  try {
    Y = renormalize(ctx, false, *mR, psi, psi);
    Z = renormalize(ctx, true, *mL, psi, psi);
  } catch (...) {
    ctx.precision = saved;
    throw;
  }
  ctx.precision = saved;
  gl = mpo_gradient(ctx, true, lmpo, lopr, *Y);
  gr = mpo_gradient(ctx, false, rmpo, ropr, *Z);
}

std::unique_ptr<DTensor> compute_merged_operator(Context& ctx, bool forward, const DTensor& mpo,
                                                 const DTensor& opr) {
  if (mpo.sh.rank != 4 || opr.sh.rank != 3) throw Error(kInvalidArgument, "merged operator: bad ranks");
  if (static_cast<int64_t>(mpo.host.size()) != mpo.nnz)
    throw Error(kInvalidArgument, "merged operator: MPO coefficients must be available on the host");
  PhaseTimer tplan(ctx, kPhMergePlan);
  // the plan depends on the layouts and on the MPO coefficients (data version)
  const MergePlan& plan = merge_plan(ctx, forward, mpo, opr);
  auto out = std::make_unique<DTensor>();
  static_cast<Tensor&>(*out) = plan.layout;
  tplan.stop();
  PhaseTimer talloc(ctx, kPhMergeAlloc);
  out->ctx = &ctx;
  out->alloc_device(ctx.stream, true);
  talloc.stop();
  PhaseTimer trun(ctx, kPhMergeRun);
  launch_scatter(plan.dst.get(), plan.ndst, plan.src.get(), opr.d, out->d, ctx.stream);
  ctx.kernel_launches += 1;
  return out;
}

// ---------------------------------------------------------------------------
// wavefunction merge / expand
// ---------------------------------------------------------------------------
WaveMerge wave_merge_infos(const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr, const DTensor& ropr) {
  auto neg = [](const std::vector<Qn>& v) {
    std::vector<Qn> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = -v[i];
    return o;
  };
  WaveMerge wm;
  wm.ql = MergeInfo({neg(lopr.sh.qshape[2]), neg(lmpo.sh.qshape[2])}, {lopr.sh.dshape[0], lmpo.sh.dshape[1]});
  wm.qr = MergeInfo({neg(rmpo.sh.qshape[2]), neg(ropr.sh.qshape[2])}, {rmpo.sh.dshape[1], ropr.sh.dshape[0]});
  return wm;
}

std::unique_ptr<WavePlan> plan_merge_wave(Context& ctx, const WaveMerge& wm, const Tensor& lwfn, const Tensor& rwfn) {
  auto wp = std::make_unique<WavePlan>();
  int K = 0;
  Shape t4 = gemm_result_shape(kNoTrans, kNoTrans, lwfn.sh, rwfn.sh, 4, &K);
  auto tasks = enumerate_gemm(kNoTrans, kNoTrans, lwfn, rwfn, t4, K);
  Tensor& psi = wp->psi;
  psi.sh.rank = 2;
  psi.sh.q = t4.q;
  psi.sh.qshape = {wm.ql.q_merged, wm.qr.q_merged};
  psi.sh.dshape = {wm.ql.d_merged, wm.qr.d_merged};
  psi.sh.finalize();
  psi.allocate_allowed();
  const int nn = t4.nsec(1), nr = t4.nsec(3);
  build_plan_impl(wp->plan, kNoTrans, kNoTrans, lwfn, rwfn, K, std::move(tasks), [&](int64_t ctag) {
    int ti[kMaxRank];
    t4.index(ctag, ti);
    const int ipr = ti[0] * nn + ti[1], ipc = ti[2] * nr + ti[3];
    const int A = wm.ql.merged_of[ipr], B = wm.qr.merged_of[ipc];
    int pi[2] = {A, B};
    const int32_t ps = psi.find(psi.sh.tag(pi));
    if (ps < 0) throw Error(kInternal, "merge_wave: psi block missing");
    const int dB = psi.sh.dshape[1][B];
    CMap m;
    m.off = psi.offsets[ps] + int64_t(wm.ql.offset_packed[ipr]) * dB + wm.qr.offset_packed[ipc];
    m.m = t4.dshape[0][ti[0]] * t4.dshape[1][ti[1]];
    m.n = t4.dshape[2][ti[2]] * t4.dshape[3][ti[3]];
    m.ldc = dB;
    return m;
  });
  wp->plan.upload(ctx.stream);
  return wp;
}

std::unique_ptr<DTensor> run_merge_wave(Context& ctx, WavePlan& wp, const DTensor& lwfn, const DTensor& rwfn) {
  auto psi = std::make_unique<DTensor>();
  static_cast<Tensor&>(*psi) = wp.psi;
  psi->ctx = &ctx;
  psi->alloc_device(ctx.stream, true);
  wp.plan.run(1.0, lwfn.d, rwfn.d, psi->d, gemm_scratch(ctx, wp.plan), ctx.stream);
  ctx.kernel_launches += 1;
  return psi;
}

std::unique_ptr<DTensor> merge_wave(Context& ctx, const WaveMerge& wm, const DTensor& lwfn, const DTensor& rwfn) {
  PhaseTimer tm(ctx, kPhWaveMerge);
  auto wp = plan_merge_wave(ctx, wm, lwfn, rwfn);
  return run_merge_wave(ctx, *wp, lwfn, rwfn);
}

static std::vector<std::vector<Qn>> split_q(const MergeInfo& info) { return info.qshape; }

std::unique_ptr<DTensor> expand_rows(Context& ctx, const MergeInfo& info, const DTensor& b) {
  // b[A, x...] -> a[(i,j), x...]  (QSTexpand, include/btas/QSPARSE/QSTmerge.h:218-295)
  const int MR = static_cast<int>(info.qshape.size());
  auto a = std::make_unique<DTensor>();
  a->sh.rank = MR + b.sh.rank - 1;
  a->sh.q = b.sh.q;
  a->sh.qshape = split_q(info);
  a->sh.dshape = info.dshape;
  for (int i = 1; i < b.sh.rank; ++i) {
    a->sh.qshape.push_back(b.sh.qshape[i]);
    a->sh.dshape.push_back(b.sh.dshape[i]);
  }
  a->sh.finalize();
  const int64_t b_stride = b.sh.rank > 1 ? b.sh.stride[0] : 1;
  const int64_t a_stride = a->sh.stride[MR - 1];
  struct Pend {
    int64_t atag, src_off;
    int rows, cols, sld;
  };
  std::vector<Pend> pend;
  int idx[kMaxRank];
  for (size_t bb = 0; bb < b.tags.size(); ++bb) {
    const int64_t i = b.tags[bb] / b_stride, j = b.tags[bb] % b_stride;
    b.sh.index(b.tags[bb], idx);
    int64_t rest = 1;
    for (int k = 1; k < b.sh.rank; ++k) rest *= b.sh.dshape[k][idx[k]];
    for (int ip : info.members[i]) {
      const int d = info.d_packed[ip];
      if (d == 0) continue;
      const int64_t at = ip * a_stride + j;
      if (!a->sh.allowed_tag(at)) continue;
      pend.push_back({at, b.offsets[bb] + int64_t(info.offset_packed[ip]) * rest, d, static_cast<int>(rest),
                      static_cast<int>(rest)});
    }
  }
  std::sort(pend.begin(), pend.end(), [](const Pend& x, const Pend& y) { return x.atag < y.atag; });
  std::vector<int64_t> tags;
  for (auto& p : pend) tags.push_back(p.atag);
  a->set_blocks(tags);
  std::vector<DCopy> cp;
  for (auto& p : pend) {
    const int32_t s = a->find(p.atag);
    cp.push_back(DCopy{a->offsets[s], p.src_off, p.rows, p.cols, p.cols, p.sld, 1.0});
  }
  a->ctx = &ctx;
  a->alloc_device(ctx.stream, false);
  DevArray<DCopy> dc;
  dc.upload(cp, ctx.stream);
  launch_copy(dc.get(), static_cast<int>(cp.size()), b.d, a->d, 0, ctx.stream);
  ctx.kernel_launches += 1;
  return a;
}

std::unique_ptr<DTensor> expand_cols(Context& ctx, const DTensor& b, const MergeInfo& info) {
  // b[x..., B] -> a[x..., (i,j)]
  const int MC = static_cast<int>(info.qshape.size());
  const int MR = b.sh.rank - 1;
  auto a = std::make_unique<DTensor>();
  a->sh.rank = MR + MC;
  a->sh.q = b.sh.q;
  for (int i = 0; i < MR; ++i) {
    a->sh.qshape.push_back(b.sh.qshape[i]);
    a->sh.dshape.push_back(b.sh.dshape[i]);
  }
  for (int i = 0; i < MC; ++i) {
    a->sh.qshape.push_back(info.qshape[i]);
    a->sh.dshape.push_back(info.dshape[i]);
  }
  a->sh.finalize();
  const int64_t b_stride = b.sh.stride[MR - 1];
  const int64_t a_stride = a->sh.stride[MR - 1];
  struct Pend {
    int64_t atag, src_off;
    int rows, cols, sld;
  };
  std::vector<Pend> pend;
  int idx[kMaxRank];
  for (size_t bb = 0; bb < b.tags.size(); ++bb) {
    const int64_t i = b.tags[bb] / b_stride, j = b.tags[bb] % b_stride;
    b.sh.index(b.tags[bb], idx);
    int64_t rows = 1;
    for (int k = 0; k < MR; ++k) rows *= b.sh.dshape[k][idx[k]];
    const int dB = b.sh.dshape[MR][idx[MR]];
    for (int ip : info.members[j]) {
      const int d = info.d_packed[ip];
      if (d == 0) continue;
      const int64_t at = i * a_stride + ip;
      if (!a->sh.allowed_tag(at)) continue;
      pend.push_back({at, b.offsets[bb] + info.offset_packed[ip], static_cast<int>(rows), d, dB});
    }
  }
  std::sort(pend.begin(), pend.end(), [](const Pend& x, const Pend& y) { return x.atag < y.atag; });
  std::vector<int64_t> tags;
  for (auto& p : pend) tags.push_back(p.atag);
  a->set_blocks(tags);
  std::vector<DCopy> cp;
  for (auto& p : pend) {
    const int32_t s = a->find(p.atag);
    cp.push_back(DCopy{a->offsets[s], p.src_off, p.rows, p.cols, p.cols, p.sld, 1.0});
  }
  a->ctx = &ctx;
  a->alloc_device(ctx.stream, false);
  DevArray<DCopy> dc;
  dc.upload(cp, ctx.stream);
  launch_copy(dc.get(), static_cast<int>(cp.size()), b.d, a->d, 0, ctx.stream);
  ctx.kernel_launches += 1;
  return a;
}

std::unique_ptr<DTensor> merge_rows(Context& ctx, const MergeInfo& info, const DTensor& a) {
  // a[(i,j), x...] -> b[A, x...]  (QSTmerge over the leading indices,
  // include/btas/QSPARSE/QSTmerge.h:31-120): every block is a contiguous row range
  const int MR = static_cast<int>(info.qshape.size());
  const int MC = a.sh.rank - MR;
  if (MC < 1) throw Error(kInvalidArgument, "merge_rows: nothing left to keep as columns");
  auto b = std::make_unique<DTensor>();
  b->sh.rank = MC + 1;
  b->sh.q = a.sh.q;
  b->sh.qshape.push_back(info.q_merged);
  b->sh.dshape.push_back(info.d_merged);
  for (int i = MR; i < a.sh.rank; ++i) {
    b->sh.qshape.push_back(a.sh.qshape[i]);
    b->sh.dshape.push_back(a.sh.dshape[i]);
  }
  b->sh.finalize();
  const int64_t a_stride = a.sh.stride[MR - 1];  // tag = packed_row * a_stride + rest
  const int64_t b_stride = b->sh.stride[0];
  struct Pend {
    int64_t btag, src_off;
    int rows, cols, roff;
  };
  std::vector<Pend> pend;
  int idx[kMaxRank];
  for (size_t ab = 0; ab < a.tags.size(); ++ab) {
    const int64_t ip = a.tags[ab] / a_stride, rest = a.tags[ab] % a_stride;
    const int A = info.merged_of[ip];
    const int64_t bt = A * b_stride + rest;
    if (!b->sh.allowed_tag(bt)) continue;
    a.sh.index(a.tags[ab], idx);
    int64_t cols = 1;
    for (int k = MR; k < a.sh.rank; ++k) cols *= a.sh.dshape[k][idx[k]];
    pend.push_back({bt, a.offsets[ab], info.d_packed[ip], static_cast<int>(cols), info.offset_packed[ip]});
  }
  std::vector<int64_t> tags;
  for (auto& p : pend) tags.push_back(p.btag);
  std::sort(tags.begin(), tags.end());
  tags.erase(std::unique(tags.begin(), tags.end()), tags.end());
  b->set_blocks(tags);
  std::vector<DCopy> cp;
  for (auto& p : pend) {
    const int32_t s = b->find(p.btag);
    cp.push_back(DCopy{b->offsets[s] + int64_t(p.roff) * p.cols, p.src_off, p.rows, p.cols, p.cols, p.cols, 1.0});
  }
  b->ctx = &ctx;
  b->alloc_device(ctx.stream, true);
  DevArray<DCopy> dc;
  dc.upload(cp, ctx.stream);
  launch_copy(dc.get(), static_cast<int>(cp.size()), a.d, b->d, 0, ctx.stream);
  ctx.kernel_launches += 1;
  return b;
}

std::unique_ptr<DTensor> merge_cols(Context& ctx, const DTensor& a, const MergeInfo& info) {
  const int MC = static_cast<int>(info.qshape.size());
  const int MR = a.sh.rank - MC;
  if (MR < 1) throw Error(kInvalidArgument, "merge_cols: nothing left to keep as rows");
  auto b = std::make_unique<DTensor>();
  b->sh.rank = MR + 1;
  b->sh.q = a.sh.q;
  for (int i = 0; i < MR; ++i) {
    b->sh.qshape.push_back(a.sh.qshape[i]);
    b->sh.dshape.push_back(a.sh.dshape[i]);
  }
  b->sh.qshape.push_back(info.q_merged);
  b->sh.dshape.push_back(info.d_merged);
  b->sh.finalize();
  const int64_t a_stride = a.sh.stride[MR - 1];
  const int64_t b_stride = b->sh.stride[MR - 1];
  struct Pend {
    int64_t btag, src_off;
    int rows, cols, coff;
  };
  std::vector<Pend> pend;
  int idx[kMaxRank];
  for (size_t ab = 0; ab < a.tags.size(); ++ab) {
    const int64_t i = a.tags[ab] / a_stride, ip = a.tags[ab] % a_stride;
    const int B = info.merged_of[ip];
    const int64_t bt = i * b_stride + B;
    if (!b->sh.allowed_tag(bt)) continue;
    a.sh.index(a.tags[ab], idx);
    int64_t rows = 1;
    for (int k = 0; k < MR; ++k) rows *= a.sh.dshape[k][idx[k]];
    pend.push_back({bt, a.offsets[ab], static_cast<int>(rows), info.d_packed[ip], info.offset_packed[ip]});
  }
  std::vector<int64_t> tags;
  for (auto& p : pend) tags.push_back(p.btag);
  std::sort(tags.begin(), tags.end());
  tags.erase(std::unique(tags.begin(), tags.end()), tags.end());
  b->set_blocks(tags);
  std::vector<DCopy> cp;
  for (auto& p : pend) {
    const int32_t s = b->find(p.btag);
    b->sh.index(p.btag, idx);
    const int dB = b->sh.dshape[MR][idx[MR]];
    cp.push_back(DCopy{b->offsets[s] + p.coff, p.src_off, p.rows, p.cols, dB, p.cols, 1.0});
  }
  b->ctx = &ctx;
  b->alloc_device(ctx.stream, true);
  DevArray<DCopy> dc;
  dc.upload(cp, ctx.stream);
  launch_copy(dc.get(), static_cast<int>(cp.size()), a.d, b->d, 0, ctx.stream);
  ctx.kernel_launches += 1;
  return b;
}

std::unique_ptr<DTensor> gemm_new(Context& ctx, Trans ta, Trans tb, double alpha, const DTensor& a, const DTensor& b,
                                  int c_rank) {
  int K = 0;
  Shape cs = gemm_result_shape(ta, tb, a.sh, b.sh, c_rank, &K);
  auto tasks = enumerate_gemm(ta, tb, a, b, cs, K);
  auto c = std::make_unique<DTensor>();
  layout_from_tasks(*c, cs, tasks);
  GemmPlan plan;
  build_gemm_plan(plan, ta, tb, a, b, *c, K, std::move(tasks));
  plan.upload(ctx.stream);
  c->ctx = &ctx;
  c->alloc_device(ctx.stream, true);
  plan.run(alpha, a.d, b.d, c->d, gemm_scratch(ctx, plan), ctx.stream);
  ctx.kernel_launches += 1;
  return c;
}

double normalize_tensor(Context& ctx, DTensor& x) {
  const int64_t n = x.nnz;
  if (n == 0) return 0.0;
  const int nblk = multidot_blocks(n);
  ctx.partial.ensure(size_t(nblk) * 100 * sizeof(double), ctx.stream);
  ctx.scalars.ensure(256 * sizeof(double), ctx.stream);
  double* sc = ctx.scalars.as<double>();
  launch_multidot(x.d, 1, x.d, 1, n, n, sc + 100, ctx.partial.as<double>(), nblk, ctx.stream);
  launch_scal_dev(x.d, n, sc + 100, 1, ctx.stream);
  ctx.kernel_launches += 3;
  double nrm2 = 0.0;
  cuda_check(cudaMemcpyAsync(&nrm2, sc + 100, sizeof(double), cudaMemcpyDeviceToHost, ctx.stream), "norm d2h");
  ctx.sync();
  return std::sqrt(nrm2);
}

// ---------------------------------------------------------------------------
// Davidson (single root)
// ---------------------------------------------------------------------------
// The Davidson loop of src/diagonalize.hpp:310-449 in the context's current
// precision.  Stops when |r|^2 < tol, or — with rel_floor > 0 — when |r|^2 falls
// below (rel_floor * E)^2, the resolution of an inexact operator.  With anchor set,
// the first H_eff * psi (of the start vector) is applied in FP64 and the rest in the
// context's precision; S.rnorm_fp64 then holds the start vector's FP64 residual.
static double davidson_run(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& diag, DTensor& wfnc,
                           double tol, double rel_floor, int max_macro, DavidsonStats& S, bool anchor = false) {
  const int max_ritz = 10;
  const int64_t n = wfnc.nnz;
  if (diag.nnz != wfnc.nnz)
    throw Error(kInvalidArgument, "diagonalize: diag and wavefunction layouts differ");
  cudaStream_t st = ctx.stream;
  SigmaPlan& sp = sigma_plan(ctx, L, R, wfnc);
  ctx.work.ensure(size_t(2 * max_ritz + 1) * std::max<int64_t>(n, 1) * sizeof(double), ctx.stream);
  double* trial = ctx.work.as<double>();
  double* sigma = trial + int64_t(max_ritz) * n;
  double* errv = sigma + int64_t(max_ritz) * n;
  const int nblk = multidot_blocks(n);
  ctx.partial.ensure(size_t(nblk) * 100 * sizeof(double), ctx.stream);
  ctx.scalars.ensure(256 * sizeof(double), ctx.stream);
  double* part = ctx.partial.as<double>();
  double* sc = ctx.scalars.as<double>();  // [0..99] dots, [100] norm, [101] dot, [128..227] rvec, [230..] roots
  double* rvec_d = sc + 128;

  PhaseTimer trest(ctx, kPhDavidsonRest);
  // Lower roots (multi-root, src/diagonalize.hpp:200-277): with s_j = <S_j|c> and
  // h_j = <H_j|c>, H' c = H c - S_j h_j - H_j s_j + E_j S_j s_j for every projected
  // root j, S_j / H_j being root j's wavefunction / H_eff times it in this basis.
  const Projection* proj = ctx.projection;
  if (proj && proj->S.size() > kMaxProjected) throw Error(kInvalidArgument, "diagonalize: too many lower roots");
  std::vector<double> pdots;
  auto project_dots = [&](const double* c) {
    const size_t np = proj->S.size();
    pdots.assign(2 * np, 0.0);
    for (size_t j = 0; j < np; ++j) {
      launch_multidot(proj->S[j], 1, c, 1, n, n, sc + 230 + 2 * j, part, nblk, st);
      launch_multidot(proj->H[j], 1, c, 1, n, n, sc + 231 + 2 * j, part, nblk, st);
      ctx.kernel_launches += 4;
    }
    cuda_check(cudaMemcpyAsync(pdots.data(), sc + 230, 2 * np * sizeof(double), cudaMemcpyDeviceToHost, st),
               "projection d2h");
    ctx.sync();
  };
  auto sigma_of = [&](int k, int precision) {
    PhaseTimer tm(ctx, precision == kFP64 && ctx.precision != kFP64 ? kPhSigmaFP64 : kPhSigma);
    cuda_check(cudaMemsetAsync(sigma + k * n, 0, n * sizeof(double), st), "sigma zero");
    sigma_run(ctx, sp, L, R, trial + k * n, sigma + k * n, precision);
    S.n_sigma += 1;
    if (precision == kFP64) S.n_sigma_fp64 += 1;
    tm.stop();
    ctx.timers[kPhDavidsonRest] -= tm.dt;  // H_eff * psi is not part of the rest
    if (proj && !proj->S.empty()) {
      project_dots(trial + k * n);
      for (size_t j = 0; j < proj->S.size(); ++j) {
        const double s = pdots[2 * j], h = pdots[2 * j + 1];
        launch_axpy(sigma + k * n, proj->S[j], n, -h + proj->E[j] * s, st);
        launch_axpy(sigma + k * n, proj->H[j], n, -s, st);
        ctx.kernel_launches += 2;
      }
    }
  };
  // c <- c - sum_j <S_j|c> S_j (before normalisation)
  auto orthogonalize_roots = [&](double* c) {
    if (!proj || proj->S.empty()) return;
    project_dots(c);
    for (size_t j = 0; j < proj->S.size(); ++j) launch_axpy(c, proj->S[j], n, -pdots[2 * j], st);
    ctx.kernel_launches += static_cast<int64_t>(proj->S.size());
  };
  auto normalize = [&](double* x) {
    launch_multidot(x, 1, x, 1, n, n, sc + 100, part, nblk, st);
    launch_scal_dev(x, n, sc + 100, 1, st);
    ctx.kernel_launches += 3;
  };

  launch_copy_vec(trial, wfnc.d, n, st);
  orthogonalize_roots(trial);
  double eval = 0.0;
  int niter = 0, iconv = 0;
  std::vector<double> hdots(100), heff, rvec, rval;
  while (iconv < 1 && niter < max_macro) {
    normalize(trial);
    sigma_of(0, anchor && niter == 0 ? kFP64 : ctx.precision);
    for (int m = 1; m <= max_ritz; ++m) {
      launch_multidot(trial, m, sigma, m, n, n, sc, part, nblk, st);
      ctx.kernel_launches += 2;
      cuda_check(cudaMemcpyAsync(hdots.data(), sc, m * m * sizeof(double), cudaMemcpyDeviceToHost, st), "heff d2h");
      ctx.sync();
      heff.assign(m * m, 0.0);
      for (int i = 0; i < m; ++i)
        for (int j = 0; j <= i; ++j) {
          const double h = hdots[i * m + j];  // trial_i . sigma_j
          heff[i * m + j] = h;
          heff[j * m + i] = h;
        }
      jacobi_eigh(m, heff, rval, rvec);  // rvec[i*m + j]: component i of eigenvector j
      eval = rval[0];
      S.micro += 1;
      upload_staged(rvec_d, rvec.data(), m * m * sizeof(double), st);
      launch_rotate(trial, m, n, n, rvec_d, m, nullptr, st);
      launch_rotate(sigma, m, n, n, rvec_d, m, nullptr, st);
      launch_copy_vec(errv, sigma, n, st);
      launch_axpy(errv, trial, n, -eval, st);
      launch_multidot(errv, 1, errv, 1, n, n, sc + 101, part, nblk, st);
      ctx.kernel_launches += 6;
      double rnorm = 0.0;
      cuda_check(cudaMemcpyAsync(&rnorm, sc + 101, sizeof(double), cudaMemcpyDeviceToHost, st), "rnorm d2h");
      ctx.sync();
      S.rnorm = rnorm;
      if (anchor && niter == 0 && m == 1) S.rnorm_fp64 = rnorm;
      if (rnorm < tol || (rel_floor > 0.0 && rnorm < rel_floor * rel_floor * eval * eval)) {
        ++iconv;
        break;
      }
      if (m < max_ritz) {
        // correction vector orthonormalised against the subspace: the reference
        // projects out one trial vector at a time (src/diagonalize.hpp:425-431); here
        // classical Gram-Schmidt is applied twice, all m projections per pass in one
        // multi-dot and one update (the same vector to rounding, 12 launches for m)
        launch_precondition(errv, diag.d, n, eval, st);
        normalize(errv);
        for (int pass = 0; pass < 2; ++pass) {
          launch_multidot(trial, m, errv, 1, n, n, sc + 104, part, nblk, st);
          launch_project_out(errv, trial, m, n, n, sc + 104, st);
          ctx.kernel_launches += 3;
        }
        normalize(errv);
        launch_copy_vec(trial + m * n, errv, n, st);
        ctx.kernel_launches += 2;
        sigma_of(m, ctx.precision);
      }
    }
    ++niter;
  }
  S.macro += niter;
  S.converged = iconv;
  launch_copy_vec(wfnc.d, trial, n, st);
  orthogonalize_roots(wfnc.d);  // multH.orthonormalize (src/diagonalize.hpp:446)
  normalize(wfnc.d);
  ctx.sync();
  return eval;
}

double diagonalize(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& diag, DTensor& wfnc, double tol,
                   DavidsonStats* stats) {
  DavidsonStats local;
  DavidsonStats& S = stats ? *stats : local;
  S = DavidsonStats{};
  if (ctx.precision == kFP64) return davidson_run(ctx, L, R, diag, wfnc, tol, 0.0, 4, S);
  // Split precision.  (1) The Davidson iterations with the tensor-core operator, to
  // its resolution.  (2) Refinement: one FP64 H_eff * psi of that vector anchors a
  // continuation of the Davidson run in which only the new correction vectors are
  // applied in split precision.  Subspace entries that involve the anchor are FP64
  // (<t_i|H|psi> = <t_i|sigma_FP64>), so the split error enters the Ritz value only
  // through the small correction components, at second order; with a start vector
  // already within the tolerance the accepted value is the FP64 Rayleigh quotient.
  // A continuation that ends unconverged (subspace full) is anchored once more.
  const double e_split = davidson_run(ctx, L, R, diag, wfnc, tol, ctx.split_floor, 4, S);
  check_device_error(ctx);
  S.energy_split = e_split;
  double e = e_split;
  for (int round = 0; round < ctx.refine_rounds; ++round) {
    DavidsonStats R1;
    e = davidson_run(ctx, L, R, diag, wfnc, tol, 0.0, 1, R1, /*anchor=*/true);
    check_device_error(ctx);
    S.n_sigma += R1.n_sigma;
    S.n_sigma_fp64 += R1.n_sigma_fp64;
    S.micro += R1.micro;
    S.macro += R1.macro;
    S.rnorm = R1.rnorm;
    S.rnorm_fp64 = R1.rnorm_fp64;
    S.converged = R1.converged;
    if (R1.converged) break;
  }
  return e;
}


// ---------------------------------------------------------------------------
// one bond
// ---------------------------------------------------------------------------

// Plans are keyed by structural layout ids and kept across bonds and sweeps (a
// converged sweep repeats the layouts of the previous one); the large packed
// operand buffers go back to the block cache after every bond.
void release_bond_buffers(Context& ctx) {
  for (auto& kv : ctx.sigma_plans) {
    for (Packed* P : {&kv.second->pk_L, &kv.second->pk_R, &kv.second->pk_psi, &kv.second->pk_scr1}) {
      P->buf.release();
      P->src_layout = 0;
      P->src_version = ~0ull;
    }
    kv.second->group_scr.release();
    kv.second->staged.release();
    kv.second->drop_graph();
  }
  if (ctx.sigma_plans.size() > ctx.max_plans) ctx.sigma_plans.clear();
  if (ctx.diag_plans.size() > ctx.max_plans) ctx.diag_plans.clear();
  if (ctx.merge_plans.size() > ctx.max_plans) ctx.merge_plans.clear();
  if (ctx.renorm_plans.size() > ctx.max_plans) ctx.renorm_plans.clear();
}

BondOut optimize_twosite_merged(Context& ctx, bool forward, const DTensor& lmpo, const DTensor& rmpo,
                                const DTensor& lopr, const DTensor& ropr, const DTensor& lwfn, const DTensor& rwfn,
                                double tole, int M, double noise) {
  BondOut out;
  double t0 = now();
  auto mL = compute_merged_operator(ctx, true, lmpo, lopr);
  auto mR = compute_merged_operator(ctx, false, rmpo, ropr);
  WaveMerge wm = wave_merge_infos(lmpo, rmpo, lopr, ropr);
  auto psi = merge_wave(ctx, wm, lwfn, rwfn);
  double t1 = now();
  out.stats.t_merge = t1 - t0;
  DTensor diag;
  static_cast<Tensor&>(diag) = static_cast<const Tensor&>(*psi);
  diag.d = nullptr;
  diag.ctx = &ctx;
  diag.alloc_device(ctx.stream, true);
  compute_diagonal_elements(ctx, *mL, *mR, diag);
  ctx.sync();
  double t2 = now();
  out.stats.t_diag = t2 - t1;
  const double f0 = ctx.sigma_flops;
  out.stats.energy = diagonalize(ctx, *mL, *mR, diag, *psi, tole, &out.stats.dav);
  out.stats.sigma_flops = ctx.sigma_flops - f0;
  double t3 = now();
  out.stats.t_davidson = t3 - t2;
  CanonResult cr = canonicalize(ctx, forward, *psi, M, noise);
  double t4 = now();
  out.stats.t_svd = t4 - t3;
  if (forward)
    out.env = renormalize(ctx, true, *mL, *cr.lmat, *cr.lmat);
  else
    out.env = renormalize(ctx, false, *mR, *cr.rmat, *cr.rmat);
  double t5 = now();
  out.stats.t_renorm = t5 - t4;
  out.lwfn = expand_rows(ctx, wm.ql, *cr.lmat);
  out.rwfn = expand_cols(ctx, *cr.rmat, wm.qr);
  release_bond_buffers(ctx);
  return out;
}

}  // namespace mpsxx
