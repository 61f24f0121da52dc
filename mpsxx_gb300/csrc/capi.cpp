// extern "C" boundary of libmpsxx_gb300 (declared in include/mpsxx_gb300.h).
#include <cstring>
#include <exception>
#include <memory>
#include <string>

#include "../../include/mpsxx_gb300.h"
#include "engine.hpp"

using namespace mpsxx;

struct mpsxx_context {
  std::unique_ptr<Context> ctx;
};
struct mpsxx_tensor {
  std::unique_ptr<DTensor> t;
  mpsxx_context* owner = nullptr;
};

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <class F>
int guard(F&& f) {
  try {
    g_last_error.clear();
    f();
    return MPSXX_OK;
  } catch (const Error& e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return fail(MPSXX_ALLOC, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(MPSXX_INTERNAL, e.what());
  }
}

void need(bool c, const char* msg) {
  if (!c) throw Error(kInvalidArgument, msg);
}

Context& ctx_of(mpsxx_context* c) {
  need(c && c->ctx, "null context");
  return *c->ctx;
}

const DTensor& ten(const mpsxx_tensor* t) {
  need(t && t->t, "null tensor");
  return *t->t;
}

DTensor& ten_mut(mpsxx_tensor* t) {
  need(t && t->t, "null tensor");
  return *t->t;
}

void need_device(const DTensor& t) { need(t.d != nullptr || t.nnz == 0, "tensor has no device storage"); }

mpsxx_tensor* wrap(std::unique_ptr<DTensor> t, mpsxx_context* owner) {
  auto* w = new mpsxx_tensor;
  w->t = std::move(t);
  w->owner = owner;
  return w;
}
}  // namespace

namespace mpsxx {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace mpsxx

extern "C" {

int mpsxx_version(void) { return 100; }

const char* mpsxx_last_error(void) { return g_last_error.c_str(); }

int mpsxx_context_create(int device, void* stream, mpsxx_context** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    auto* c = new mpsxx_context;
    try {
      c->ctx = std::make_unique<Context>(device, static_cast<cudaStream_t>(stream));
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

int mpsxx_context_destroy(mpsxx_context* ctx) {
  return guard([&] { delete ctx; });
}

int mpsxx_context_sync(mpsxx_context* ctx) {
  return guard([&] { ctx_of(ctx).sync(); });
}

int mpsxx_context_set_precision(mpsxx_context* ctx, int precision) {
  return guard([&] {
    need(precision == MPSXX_FP64 || precision == MPSXX_SPLIT_TF32 || precision == MPSXX_SPLIT_TF32_ALL,
         "unknown precision");
    ctx_of(ctx).precision = precision;
  });
}

int mpsxx_context_get_precision(const mpsxx_context* ctx, int* precision) {
  return guard([&] {
    need(ctx && ctx->ctx && precision, "null argument");
    *precision = ctx->ctx->precision;
  });
}

int mpsxx_context_set_truncation(mpsxx_context* ctx, double tie_rtol) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    ctx->ctx->tie_rtol = tie_rtol;
  });
}

int mpsxx_context_set_split_refinement(mpsxx_context* ctx, double residual_floor, int rounds) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    need(rounds <= 64, "mpsxx_context_set_split_refinement: at most 64 rounds");
    ctx->ctx->split_floor = residual_floor >= 0.0 ? residual_floor : mpsxx::kSplitResidualFloorDefault;
    ctx->ctx->refine_rounds = rounds >= 0 ? rounds : mpsxx::kRefineRoundsDefault;
  });
}

int mpsxx_context_counters(const mpsxx_context* ctx, int64_t* launches, double* sigma_flops, int64_t* sigma_calls) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    if (launches) *launches = ctx->ctx->kernel_launches;
    if (sigma_flops) *sigma_flops = ctx->ctx->sigma_flops;
    if (sigma_calls) *sigma_calls = ctx->ctx->sigma_calls;
  });
}

int mpsxx_context_profile(mpsxx_context* ctx, int enable, int reset, double* t, int n, int* count) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    mpsxx::Context& c = *ctx->ctx;
    if (count) *count = mpsxx::kNumPhases;
    for (int i = 0; t && i < n && i < mpsxx::kNumPhases; ++i) t[i] = c.timers[i];
    if (reset)
      for (double& x : c.timers) x = 0.0;
    if (enable >= 0) c.profile = enable != 0;
  });
}

int mpsxx_context_set_sigma_schedule(mpsxx_context* ctx, int64_t w_budget_bytes, int target_tiles,
                                     int fp32_intermediate) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    need(target_tiles >= 0, "negative tile target");
    Context& c = *ctx->ctx;
    c.sigma_w_budget = w_budget_bytes;
    c.sigma_target_tiles = target_tiles;
    c.sigma_fp32_intermediate = fp32_intermediate != 0;
    c.sigma_plans.clear();  // plans are rebuilt (and scheduled) on next use
  });
}

int mpsxx_context_set_sigma_operator_format(mpsxx_context* ctx, int fp32_operators) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    Context& c = *ctx->ctx;
    c.sigma_fp32_operators = fp32_operators != 0;
    c.sigma_plans.clear();  // plans are rebuilt with the new packing on next use
  });
}

int mpsxx_context_set_device_timeout(mpsxx_context* ctx, int64_t timeout_ns) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    ctx->ctx->device_timeout_ns = timeout_ns > 0 ? static_cast<uint64_t>(timeout_ns) : kPkTimeoutNs;
  });
}

int mpsxx_context_set_plan_cache(mpsxx_context* ctx, int64_t max_plans) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    need(max_plans > 0, "plan cache size must be positive");
    ctx->ctx->max_plans = static_cast<size_t>(max_plans);
  });
}

int mpsxx_context_set_svd_routes(mpsxx_context* ctx, int jacobi_max_cols, int gram_max_dim) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    ctx->ctx->svd_jacobi_cols = jacobi_max_cols;
    ctx->ctx->svd_gram_max = gram_max_dim;
  });
}

int mpsxx_context_tuning(const mpsxx_context* ctx, double* out, int n, int* count) {
  return guard([&] {
    need(ctx && ctx->ctx, "null context");
    const auto& t = ctx->ctx->last_tuning;
    if (count) *count = static_cast<int>(t.size());
    for (int i = 0; out && i < n && i < static_cast<int>(t.size()); ++i) out[i] = t[i];
  });
}

int mpsxx_tensor_create(mpsxx_context* ctx, int rank, const int* q, const int* nsec, const int* qn, const int* dims,
                        int64_t nblocks, const int64_t* tags, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    need(rank >= 1 && rank <= kMaxRank, "tensor rank out of range");
    need(q && nsec && qn && dims, "null shape argument");
    auto t = std::make_unique<DTensor>();
    t->sh.rank = rank;
    t->sh.q = Qn{q[0], q[1]};
    int pos = 0;
    for (int i = 0; i < rank; ++i) {
      need(nsec[i] >= 0, "negative sector count");
      std::vector<Qn> qs;
      std::vector<int> ds;
      for (int j = 0; j < nsec[i]; ++j, ++pos) {
        qs.push_back(Qn{qn[2 * pos], qn[2 * pos + 1]});
        need(dims[pos] >= 0, "negative sector dimension");
        ds.push_back(dims[pos]);
      }
      t->sh.qshape.push_back(qs);
      t->sh.dshape.push_back(ds);
    }
    t->sh.finalize();
    if (nblocks < 0) {
      t->allocate_allowed();
    } else {
      need(nblocks == 0 || tags != nullptr, "null tags");
      t->set_blocks(std::vector<int64_t>(tags, tags + nblocks));
    }
    if (ctx) {
      Context& c = ctx_of(ctx);
      t->ctx = &c;
      t->alloc_device(c.stream, true);
      c.sync();
    }
    *out = wrap(std::move(t), ctx);
  });
}

int mpsxx_tensor_create_like(mpsxx_context* ctx, const mpsxx_tensor* like, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    const DTensor& l = ten(like);
    Context& c = ctx_of(ctx);
    auto t = std::make_unique<DTensor>();
    static_cast<Tensor&>(*t) = static_cast<const Tensor&>(l);
    t->d = nullptr;
    t->own = false;
    t->ctx = &c;
    t->alloc_device(c.stream, true);
    c.sync();
    *out = wrap(std::move(t), ctx);
  });
}

int mpsxx_tensor_destroy(mpsxx_tensor* t) {
  return guard([&] { delete t; });
}

int mpsxx_tensor_info(const mpsxx_tensor* t, int* rank, int* q, int64_t* nblocks, int64_t* nnz) {
  return guard([&] {
    const DTensor& x = ten(t);
    if (rank) *rank = x.sh.rank;
    if (q) {
      q[0] = x.sh.q.p;
      q[1] = x.sh.q.s;
    }
    if (nblocks) *nblocks = static_cast<int64_t>(x.tags.size());
    if (nnz) *nnz = x.nnz;
  });
}

int mpsxx_tensor_shape(const mpsxx_tensor* t, int* nsec, int* qn, int* dims) {
  return guard([&] {
    const DTensor& x = ten(t);
    int pos = 0;
    for (int i = 0; i < x.sh.rank; ++i) {
      if (nsec) nsec[i] = x.sh.nsec(i);
      for (int j = 0; j < x.sh.nsec(i); ++j, ++pos) {
        if (qn) {
          qn[2 * pos] = x.sh.qshape[i][j].p;
          qn[2 * pos + 1] = x.sh.qshape[i][j].s;
        }
        if (dims) dims[pos] = x.sh.dshape[i][j];
      }
    }
  });
}

int mpsxx_tensor_blocks(const mpsxx_tensor* t, int64_t* tags, int64_t* offsets) {
  return guard([&] {
    const DTensor& x = ten(t);
    for (size_t b = 0; b < x.tags.size(); ++b) {
      if (tags) tags[b] = x.tags[b];
      if (offsets) offsets[b] = x.offsets[b];
    }
  });
}

int mpsxx_tensor_upload(mpsxx_tensor* t, const double* host) {
  return guard([&] {
    DTensor& x = ten_mut(t);
    need(host != nullptr || x.nnz == 0, "null host buffer");
    // MPO site tensors (rank 4) keep a host copy: their scalar blocks are the
    // coefficients of the merged-operator scatter plans
    if (x.sh.rank == 4 || !x.ctx) x.host.assign(host, host + x.nnz);
    x.data_version = next_data_version();  // device copies of the old data (packed operands) are stale
    if (x.ctx) {
      need_device(x);
      if (x.nnz)
        cuda_check(cudaMemcpyAsync(x.d, host, x.nnz * sizeof(double), cudaMemcpyHostToDevice, x.ctx->stream), "upload");
      x.ctx->sync();
    }
  });
}

int mpsxx_tensor_download(const mpsxx_tensor* t, double* host) {
  return guard([&] {
    const DTensor& x = ten(t);
    need(host != nullptr || x.nnz == 0, "null host buffer");
    if (!x.ctx) {
      need(static_cast<int64_t>(x.host.size()) == x.nnz, "host-only tensor has no data");
      std::memcpy(host, x.host.data(), x.nnz * sizeof(double));
      return;
    }
    if (x.nnz)
      cuda_check(cudaMemcpyAsync(host, x.d, x.nnz * sizeof(double), cudaMemcpyDeviceToHost, x.ctx->stream), "download");
    x.ctx->sync();
  });
}

int mpsxx_tensor_device_ptr(const mpsxx_tensor* t, double** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    *out = ten(t).d;
  });
}

int mpsxx_gemm_tasks(int transa, int transb, const mpsxx_tensor* a, const mpsxx_tensor* b, int c_rank,
                     int64_t* ntasks, int64_t* npairs, int64_t* c_tags, int64_t* pair_ptr, int64_t* a_tags,
                     int64_t* b_tags) {
  return guard([&] {
    const DTensor& A = ten(a);
    const DTensor& B = ten(b);
    int K = 0;
    const Trans ta = transa ? kTrans : kNoTrans, tb = transb ? kTrans : kNoTrans;
    Shape c = gemm_result_shape(ta, tb, A.sh, B.sh, c_rank, &K);
    auto tasks = enumerate_gemm(ta, tb, A, B, c, K);
    int64_t np = 0;
    for (const auto& t : tasks) np += static_cast<int64_t>(t.pairs.size());
    if (ntasks) *ntasks = static_cast<int64_t>(tasks.size());
    if (npairs) *npairs = np;
    if (!c_tags) return;
    need(pair_ptr && a_tags && b_tags, "null output arrays");
    int64_t p = 0;
    for (size_t i = 0; i < tasks.size(); ++i) {
      c_tags[i] = tasks[i].c_tag;
      pair_ptr[i] = p;
      for (const auto& pr : tasks[i].pairs) {
        a_tags[p] = pr.a_tag;
        b_tags[p] = pr.b_tag;
        ++p;
      }
    }
    pair_ptr[tasks.size()] = p;
  });
}

int mpsxx_compute_sigma_vector(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                               const mpsxx_tensor* wfn, mpsxx_tensor* sgv) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    const DTensor &L = ten(lopr), &R = ten(ropr), &P = ten(wfn);
    DTensor& S = ten_mut(sgv);
    need_device(L);
    need_device(R);
    need_device(P);
    need_device(S);
    compute_sigma_vector(c, L, R, P, S);
    c.sync();
    if (c.precision != kFP64) check_device_error(c);
  });
}

namespace {
// the reference's allocate-or-accumulate contract for sgv0 (include/btas/QSPARSE/QSTBLAS.h:201-211)
void deliver(mpsxx_context* ctx, std::unique_ptr<DTensor> r, mpsxx_tensor** sgv) {
  Context& c = ctx_of(ctx);
  if (!*sgv) {
    c.sync();
    *sgv = wrap(std::move(r), ctx);
    return;
  }
  DTensor& S = ten_mut(*sgv);
  need_device(S);
  accumulate_into(c, 1.0, *r, (*sgv)->t);
  c.sync();
}
}  // namespace

int mpsxx_compute_sigma_vector_onesite(mpsxx_context* ctx, const mpsxx_tensor* mpo, const mpsxx_tensor* lopr,
                                       const mpsxx_tensor* ropr, const mpsxx_tensor* wfn, mpsxx_tensor** sgv) {
  return guard([&] {
    need(sgv != nullptr, "null output");
    Context& c = ctx_of(ctx);
    need_device(ten(lopr));
    need_device(ten(ropr));
    need_device(ten(wfn));
    deliver(ctx, sigma_onesite(c, ten(mpo), ten(lopr), ten(ropr), ten(wfn)), sgv);
    if (c.precision != kFP64) check_device_error(c);
  });
}

int mpsxx_compute_sigma_vector_twosite(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                                       const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* wfn,
                                       mpsxx_tensor** sgv) {
  return guard([&] {
    need(sgv != nullptr, "null output");
    Context& c = ctx_of(ctx);
    need_device(ten(lopr));
    need_device(ten(ropr));
    need_device(ten(wfn));
    deliver(ctx, sigma_twosite(c, ten(lmpo), ten(rmpo), ten(lopr), ten(ropr), ten(wfn)), sgv);
    if (c.precision != kFP64) check_device_error(c);
  });
}

int mpsxx_compute_sigma_vector_overlap(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                       const mpsxx_tensor* wfn, mpsxx_tensor** sgv) {
  return guard([&] {
    need(sgv != nullptr, "null output");
    Context& c = ctx_of(ctx);
    need_device(ten(lopr));
    need_device(ten(ropr));
    need_device(ten(wfn));
    deliver(ctx, sigma_overlap(c, ten(lopr), ten(ropr), ten(wfn)), sgv);
  });
}

int mpsxx_renormalize_mpo(mpsxx_context* ctx, int forward, const mpsxx_tensor* mpo, const mpsxx_tensor* opr0,
                          const mpsxx_tensor* bra, const mpsxx_tensor* ket, mpsxx_tensor** opr1) {
  return guard([&] {
    need(opr1 != nullptr, "null output");
    Context& c = ctx_of(ctx);
    need_device(ten(opr0));
    need_device(ten(bra));
    need_device(ten(ket));
    deliver(ctx, renormalize_mpo(c, forward != 0, ten(mpo), ten(opr0), ten(bra), ten(ket)), opr1);
  });
}

int mpsxx_renormalize_overlap(mpsxx_context* ctx, int forward, const mpsxx_tensor* sov0, const mpsxx_tensor* bra,
                              const mpsxx_tensor* ket, mpsxx_tensor** sov1) {
  return guard([&] {
    need(sov1 != nullptr, "null output");
    Context& c = ctx_of(ctx);
    need_device(ten(sov0));
    need_device(ten(bra));
    need_device(ten(ket));
    deliver(ctx, renormalize_overlap(c, forward != 0, ten(sov0), ten(bra), ten(ket)), sov1);
  });
}

int mpsxx_compute_guesswave(mpsxx_context* ctx, int forward, const mpsxx_tensor* mps0, const mpsxx_tensor* wfn0,
                            const mpsxx_tensor* mps1, mpsxx_tensor** wfn1) {
  return guard([&] {
    need(wfn1 != nullptr, "null output");
    Context& c = ctx_of(ctx);
    need_device(ten(mps0));
    need_device(ten(wfn0));
    need_device(ten(mps1));
    deliver(ctx, guesswave(c, forward != 0, ten(mps0), ten(wfn0), ten(mps1)), wfn1);
  });
}

int mpsxx_compute_diagonal_elements_onesite(mpsxx_context* ctx, const mpsxx_tensor* mpo, const mpsxx_tensor* lopr,
                                            const mpsxx_tensor* ropr, mpsxx_tensor* diag) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    need_device(ten(lopr));
    need_device(ten(ropr));
    need_device(ten(diag));
    auto d = diagonal_onesite(c, ten(mpo), ten(lopr), ten(ropr), ten(diag));
    // btas::Copy(scr, diag, 1): diag holds exactly the computed blocks its quantum
    // numbers allow; what it held before is dropped
    c.sync();
    diag->t = std::move(d);
  });
}

int mpsxx_compute_diagonal_elements_twosite(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                                            const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, mpsxx_tensor* diag) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    need_device(ten(lopr));
    need_device(ten(ropr));
    need_device(ten(diag));
    auto d = diagonal_twosite(c, ten(lmpo), ten(rmpo), ten(lopr), ten(ropr), ten(diag));
    // btas::Copy(scr, diag, 1): diag holds exactly the computed blocks its quantum
    // numbers allow; what it held before is dropped
    c.sync();
    diag->t = std::move(d);
  });
}

int mpsxx_sigma_plan_stats(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                           const mpsxx_tensor* wfn, double* out, int n, int* count) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    need(out != nullptr || n == 0, "null output");
    const std::vector<double> v = sigma_plan_stats(c, ten(lopr), ten(ropr), ten(wfn));
    for (int i = 0; i < n && i < static_cast<int>(v.size()); ++i) out[i] = v[i];
    if (count) *count = static_cast<int>(v.size());
  });
}

int mpsxx_compute_diagonal_elements(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                    mpsxx_tensor* diag) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    const DTensor &L = ten(lopr), &R = ten(ropr);
    DTensor& D = ten_mut(diag);
    need_device(L);
    need_device(R);
    need_device(D);
    compute_diagonal_elements(c, L, R, D);
    c.sync();
  });
}

int mpsxx_renormalize(mpsxx_context* ctx, int forward, const mpsxx_tensor* opr0, const mpsxx_tensor* bra,
                      const mpsxx_tensor* ket, mpsxx_tensor** opr1) {
  return guard([&] {
    need(opr1 != nullptr, "null output");
    Context& c = ctx_of(ctx);
    auto r = renormalize(c, forward != 0, ten(opr0), ten(bra), ten(ket));
    c.sync();
    *opr1 = wrap(std::move(r), ctx);
  });
}

int mpsxx_compute_merged_operator(mpsxx_context* ctx, int forward, const mpsxx_tensor* mpo,
                                  const mpsxx_tensor* opr, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    Context& c = ctx_of(ctx);
    auto r = compute_merged_operator(c, forward != 0, ten(mpo), ten(opr));
    c.sync();
    *out = wrap(std::move(r), ctx);
  });
}

int mpsxx_diagonalize(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                      const mpsxx_tensor* diag, mpsxx_tensor* wfnc, double tol, double* energy, int* stats) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    DavidsonStats st;
    const double e = diagonalize(c, ten(lopr), ten(ropr), ten(diag), ten_mut(wfnc), tol, &st);
    if (energy) *energy = e;
    if (stats) {
      stats[0] = st.n_sigma;
      stats[1] = st.macro;
      stats[2] = st.micro;
      stats[3] = st.converged;
    }
  });
}

int mpsxx_diagonalize_projected(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                const mpsxx_tensor* diag, mpsxx_tensor* wfnc, double tol, int nproj,
                                const mpsxx_tensor* const* S, const mpsxx_tensor* const* H, const double* E,
                                double* energy, int* stats) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    need(nproj >= 0 && (nproj == 0 || (S && H && E)), "bad projection arguments");
    const DTensor& w = ten_mut(wfnc);
    Projection proj;
    for (int j = 0; j < nproj; ++j) {
      const DTensor& s = ten(S[j]);
      const DTensor& h = ten(H[j]);
      need(s.layout_id == w.layout_id && h.layout_id == w.layout_id,
           "projected roots must have the wavefunction's block layout");
      need_device(s);
      need_device(h);
      proj.S.push_back(s.d);
      proj.H.push_back(h.d);
      proj.E.push_back(E[j]);
    }
    c.projection = &proj;
    DavidsonStats st;
    double e = 0.0;
    try {
      e = diagonalize(c, ten(lopr), ten(ropr), ten(diag), ten_mut(wfnc), tol, &st);
    } catch (...) {
      c.projection = nullptr;
      throw;
    }
    c.projection = nullptr;
    if (energy) *energy = e;
    if (stats) {
      stats[0] = st.n_sigma;
      stats[1] = st.macro;
      stats[2] = st.micro;
      stats[3] = st.converged;
    }
  });
}

int mpsxx_tensor_accumulate(mpsxx_context* ctx, double alpha, const mpsxx_tensor* x, mpsxx_tensor* y) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    const DTensor& X = ten(x);
    DTensor& Y = ten_mut(y);
    need(X.sh.rank == Y.sh.rank && X.sh.q == Y.sh.q, "accumulate: tensors of different shapes");
    for (int i = 0; i < X.sh.rank; ++i)
      need(X.sh.qshape[i] == Y.sh.qshape[i] && X.sh.dshape[i] == Y.sh.dshape[i],
           "accumulate: tensors of different sectors");
    need_device(X);
    need_device(Y);
    std::vector<DCopy> cp;
    for (size_t b = 0; b < X.tags.size(); ++b) {
      const int32_t s = Y.find(X.tags[b]);
      need(s >= 0, "accumulate: a block of x is not stored in y");
      const int64_t sz = X.block_size(static_cast<int32_t>(b));
      if (sz > 0) cp.push_back(DCopy{Y.offsets[s], X.offsets[b], 1, static_cast<int>(sz), 0, 0, alpha});
    }
    DevArray<DCopy> dc;
    dc.upload(cp, c.stream);
    launch_copy(dc.get(), static_cast<int>(cp.size()), X.d, Y.d, 1, c.stream);
    c.kernel_launches += 1;
    c.sync();
  });
}

int mpsxx_canonicalize(mpsxx_context* ctx, int forward, const mpsxx_tensor* wfnc, int M, double noise,
                       mpsxx_tensor** lmat, mpsxx_tensor** rmat) {
  return guard([&] {
    need(lmat && rmat, "null output");
    Context& c = ctx_of(ctx);
    CanonResult r = canonicalize(c, forward != 0, ten(wfnc), M, noise);
    c.sync();
    *lmat = wrap(std::move(r.lmat), ctx);
    *rmat = wrap(std::move(r.rmat), ctx);
  });
}

int mpsxx_make_noise(mpsxx_context* ctx, mpsxx_tensor* wfnc, double noise) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    DTensor& x = ten_mut(wfnc);
    need_device(x);
    std::unique_ptr<DTensor> n = make_noise(c, x, noise);
    if (!n) return;
    c.sync();
    wfnc->t = std::move(n);
  });
}

int mpsxx_noise_sequence(int64_t n, double* out) {
  return guard([&] {
    need(n >= 0 && (n == 0 || out), "invalid noise sequence request");
    const std::vector<double> seq = noise_sequence(n);
    if (n) std::memcpy(out, seq.data(), static_cast<size_t>(n) * sizeof(double));
  });
}

int mpsxx_optimize_twosite_merged(mpsxx_context* ctx, int forward, const mpsxx_tensor* lmpo,
                                  const mpsxx_tensor* rmpo, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                  const mpsxx_tensor* lwfn, const mpsxx_tensor* rwfn, double tole, int M,
                                  double noise, double* energy, mpsxx_tensor** env, mpsxx_tensor** new_lwfn,
                                  mpsxx_tensor** new_rwfn, double* stats) {
  return guard([&] {
    need(env && new_lwfn && new_rwfn, "null output");
    Context& c = ctx_of(ctx);
    BondOut b = optimize_twosite_merged(c, forward != 0, ten(lmpo), ten(rmpo), ten(lopr), ten(ropr), ten(lwfn),
                                        ten(rwfn), tole, M, noise);
    c.sync();
    if (energy) *energy = b.stats.energy;
    if (stats) {
      stats[0] = b.stats.dav.n_sigma;
      stats[1] = b.stats.sigma_flops;
      stats[2] = b.stats.t_merge;
      stats[3] = b.stats.t_diag;
      stats[4] = b.stats.t_davidson;
      stats[5] = b.stats.t_svd;
      stats[6] = b.stats.t_renorm;
      stats[7] = b.stats.dav.converged;
      stats[8] = b.stats.dav.rnorm;
      stats[9] = b.stats.dav.energy_split;
      stats[10] = b.stats.dav.rnorm_fp64;
      stats[11] = b.stats.dav.n_sigma_fp64;
    }
    *env = wrap(std::move(b.env), ctx);
    *new_lwfn = wrap(std::move(b.lwfn), ctx);
    *new_rwfn = wrap(std::move(b.rwfn), ctx);
  });
}

int mpsxx_optimize_twosite_merged_batch(mpsxx_context* ctx, int n, const int* forward,
                                        const mpsxx_tensor* const* lmpo, const mpsxx_tensor* const* rmpo,
                                        const mpsxx_tensor* const* lopr, const mpsxx_tensor* const* ropr,
                                        const mpsxx_tensor* const* lwfn, const mpsxx_tensor* const* rwfn, double tole,
                                        const int* M, const double* noise, double* energy, mpsxx_tensor** env,
                                        mpsxx_tensor** new_lwfn, mpsxx_tensor** new_rwfn, double* stats) {
  return guard([&] {
    need(n >= 0, "negative batch size");
    need(n == 0 || (forward && lmpo && rmpo && lopr && ropr && lwfn && rwfn && M && energy && env && new_lwfn &&
                    new_rwfn),
         "null argument");
    Context& c = ctx_of(ctx);
    std::vector<BondArgs> args(n);
    for (int i = 0; i < n; ++i) {
      args[i].forward = forward[i] != 0;
      args[i].lmpo = &ten(lmpo[i]);
      args[i].rmpo = &ten(rmpo[i]);
      args[i].lopr = &ten(lopr[i]);
      args[i].ropr = &ten(ropr[i]);
      args[i].lwfn = &ten(lwfn[i]);
      args[i].rwfn = &ten(rwfn[i]);
      args[i].M = M[i];
      args[i].noise = noise ? noise[i] : 0.0;
    }
    std::vector<BondOut> out = optimize_twosite_merged_batch(c, args, tole);
    for (int i = 0; i < n; ++i) {
      energy[i] = out[i].stats.energy;
      env[i] = wrap(std::move(out[i].env), ctx);
      new_lwfn[i] = wrap(std::move(out[i].lwfn), ctx);
      new_rwfn[i] = wrap(std::move(out[i].rwfn), ctx);
      if (stats) {
        const DavidsonStats& d = out[i].stats.dav;
        double* s = stats + 6 * i;
        s[0] = d.n_sigma;
        s[1] = d.n_sigma_fp64;
        s[2] = d.micro;
        s[3] = d.converged;
        s[4] = d.rnorm;
        s[5] = d.energy_split;
      }
    }
  });
}

int mpsxx_mpo_gradient(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                       const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* psi, double* grad_l,
                       double* grad_r) {
  return guard([&] {
    need(grad_l && grad_r, "null output");
    Context& c = ctx_of(ctx);
    std::vector<double> gl, gr;
    bond_mpo_gradient(c, ten(lmpo), ten(rmpo), ten(lopr), ten(ropr), ten(psi), gl, gr);
    std::memcpy(grad_l, gl.data(), gl.size() * sizeof(double));
    std::memcpy(grad_r, gr.data(), gr.size() * sizeof(double));
  });
}

int mpsxx_merge_cols(mpsxx_context* ctx, const mpsxx_tensor* a, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    Context& c = ctx_of(ctx);
    const DTensor& A = ten(a);
    need(A.sh.rank >= 3, "merge_cols: expects a tensor of 3 or more indices");
    const int r = A.sh.rank;
    MergeInfo info({A.sh.qshape[r - 2], A.sh.qshape[r - 1]}, {A.sh.dshape[r - 2], A.sh.dshape[r - 1]});
    *out = wrap(merge_cols(c, A, info), ctx);
    c.sync();
  });
}

int mpsxx_merge_rows(mpsxx_context* ctx, const mpsxx_tensor* a, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    Context& c = ctx_of(ctx);
    const DTensor& A = ten(a);
    need(A.sh.rank >= 3, "merge_rows: expects a tensor of 3 or more indices");
    MergeInfo info({A.sh.qshape[0], A.sh.qshape[1]}, {A.sh.dshape[0], A.sh.dshape[1]});
    *out = wrap(merge_rows(c, info, A), ctx);
    c.sync();
  });
}

int mpsxx_expand_rows(mpsxx_context* ctx, const mpsxx_tensor* b, const mpsxx_tensor* like, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    Context& c = ctx_of(ctx);
    const DTensor& L = ten(like);
    need(L.sh.rank == 3, "expand_rows: `like` must be a 3-index tensor");
    MergeInfo info({L.sh.qshape[0], L.sh.qshape[1]}, {L.sh.dshape[0], L.sh.dshape[1]});
    *out = wrap(expand_rows(c, info, ten(b)), ctx);
    c.sync();
  });
}

int mpsxx_gemm(mpsxx_context* ctx, int transa, int transb, double alpha, const mpsxx_tensor* a,
               const mpsxx_tensor* b, int c_rank, mpsxx_tensor** c) {
  return guard([&] {
    need(c != nullptr, "null output");
    Context& cx = ctx_of(ctx);
    *c = wrap(gemm_new(cx, transa ? kTrans : kNoTrans, transb ? kTrans : kNoTrans, alpha, ten(a), ten(b), c_rank),
              ctx);
    cx.sync();
  });
}

int mpsxx_expand_cols(mpsxx_context* ctx, const mpsxx_tensor* b, const mpsxx_tensor* like, mpsxx_tensor** out) {
  return guard([&] {
    need(out != nullptr, "null output");
    Context& c = ctx_of(ctx);
    const DTensor& L = ten(like);
    need(L.sh.rank == 3, "expand_cols: `like` must be a 3-index tensor");
    MergeInfo info({L.sh.qshape[1], L.sh.qshape[2]}, {L.sh.dshape[1], L.sh.dshape[2]});
    *out = wrap(expand_cols(c, ten(b), info), ctx);
    c.sync();
  });
}

int mpsxx_normalize(mpsxx_context* ctx, mpsxx_tensor* x, double* norm) {
  return guard([&] {
    Context& c = ctx_of(ctx);
    const double n = normalize_tensor(c, ten_mut(x));
    if (norm) *norm = n;
  });
}

int mpsxx_merge_wavefunction(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                             const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* lwfn,
                             const mpsxx_tensor* rwfn, mpsxx_tensor** psi) {
  return guard([&] {
    need(psi != nullptr, "null output");
    Context& c = ctx_of(ctx);
    WaveMerge wm = wave_merge_infos(ten(lmpo), ten(rmpo), ten(lopr), ten(ropr));
    *psi = wrap(merge_wave(c, wm, ten(lwfn), ten(rwfn)), ctx);
    c.sync();
  });
}

int mpsxx_expand_wavefunction(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                              const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* lmat,
                              const mpsxx_tensor* rmat, mpsxx_tensor** lwfn, mpsxx_tensor** rwfn) {
  return guard([&] {
    need(lwfn && rwfn, "null output");
    Context& c = ctx_of(ctx);
    WaveMerge wm = wave_merge_infos(ten(lmpo), ten(rmpo), ten(lopr), ten(ropr));
    *lwfn = wrap(expand_rows(c, wm.ql, ten(lmat)), ctx);
    *rwfn = wrap(expand_cols(c, ten(rmat), wm.qr), ctx);
    c.sync();
  });
}


int mpsxx_sigma_device_time(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                            const mpsxx_tensor* wfn, mpsxx_tensor* sgv, int reps, double* seconds) {
  return guard([&] {
    need(reps > 0 && seconds != nullptr, "bad arguments");
    Context& c = ctx_of(ctx);
    *seconds = sigma_device_time(c, ten(lopr), ten(ropr), ten(wfn), ten_mut(sgv), reps);
  });
}

}  // extern "C"
