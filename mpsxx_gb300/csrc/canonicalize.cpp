// canonicalize: per-block SVD of a merged wavefunction, global top-M truncation, and
// the split into a left- or right-normalised factor and the rest
// (src/canonicalize.hpp:88-106, QSPARSE/QSTLAPACK.h:121-288).  The blocks of one or
// many jobs (the bonds of a batched step) are routed to three SVD paths that run
// together: a batched one-sided Jacobi kernel for small blocks, a batched symmetric
// eigensolver on Gram matrices for blocks whose padded size is shared by many, and
// concurrent solver lanes (stream + host thread + cuSOLVER handle each) for the rest.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <iterator>
#include <map>
#include <random>
#include <thread>

#include "engine.hpp"

namespace mpsxx {

// ---------------------------------------------------------------------------
// canonicalize: per-block SVD, global top-M truncation, Dimm
// ---------------------------------------------------------------------------
std::vector<int> select_kept(const std::vector<std::vector<double>>& svals, int M, double tie_rtol,
                             double* discarded) {
  std::vector<double> all;
  for (const auto& v : svals) all.insert(all.end(), v.begin(), v.end());
  std::sort(all.rbegin(), all.rend());
  double cutoff = 1.0e-16;
  if (M > 0 && static_cast<size_t>(M) < all.size()) cutoff = all[M - 1] * (1.0 - tie_rtol);
  std::vector<int> kept(svals.size(), 0);
  double dn = 0.0;
  for (size_t s = 0; s < svals.size(); ++s) {
    int k = 0;
    while (k < static_cast<int>(svals[s].size()) && svals[s][k] >= cutoff) ++k;
    kept[s] = k;
    for (size_t x = k; x < svals[s].size(); ++x) dn += svals[s][x] * svals[s][x];
  }
  if (discarded) *discarded = dn;
  return kept;
}

// Default tie window of the truncation cutoff: symmetry-related singular values
// (e.g. of the (N, Sz) and (N, -Sz) sectors of an Sz = 0 state) agree to rounding
// and are kept or dropped together.
constexpr double kTieRtolDefault = 1.0e-10;
// concurrent SVD lanes of canonicalize
constexpr int kSvdLanes = 8;
// smallest min(m, n) of a block that takes the reduced-density-matrix route
constexpr int kEighMin = 96;
// largest min(m, n) of a block given to the Jacobi kernel: its cost grows as
// min(m,n)^2 max(m,n) per sweep on the FP64 pipe of one SM, which on this GPU is
// ~8 GFLOP/s; measured on the 64-chain scan, limits of 64 and 128 columns made the
// canonicalize phase 2.7x slower than the solver lanes, so only tiny blocks go there
constexpr int kJacobiUseCols = 24;
// blocks up to this many columns take the Jacobi kernel even where the batched
// eigensolver could take them (measured on the 64-chain scan: 12 beats 8, 16 and 24)
constexpr int kJacobiFirstCols = 12;
// largest Gram dimension (rows of the block for a forward step, columns backward) of
// the batched eigensolver route; larger blocks take syevd on the lanes
constexpr int kGramBatchMax = 256;
// fewest Gram matrices of one padded size that take the batched eigensolver; smaller
// groups (a single bond's few blocks of each size) are faster on the solver lanes
constexpr int kGramMinBatch = 6;

std::vector<CanonResult> canonicalize_many(Context& ctx, const std::vector<CanonJob>& jobs) {
  for (const CanonJob& jb : jobs)
    if (jb.wfnc->sh.rank != 2) throw Error(kInvalidArgument, "canonicalize: expects a merged (2-index) wavefunction");
  cudaStream_t st = ctx.stream;
  PhaseTimer tsolve(ctx, kPhSvdSolve);
  struct Blk {
    int job;
    const double* a;  // the block's data
    int32_t slot;
    int i, j, m, n, k;
    int64_t u_off, s_off, v_off;  // inside svd_mats
    bool eigh = false;            // density-matrix route: U (forward) or V (backward) from eigh,
                                  // the other factor stored already multiplied by s
    bool jacobi = false;          // batched one-sided Jacobi kernel (small blocks)
    bool gram = false;            // batched eigensolver route (implies eigh)
  };
  std::vector<Blk> blks;
  int64_t nsv = 0;  // singular values first (one contiguous read-back), then U and V^T
  int64_t maxmn = 0;
  for (size_t jb = 0; jb < jobs.size(); ++jb) {
    const DTensor& wfnc = *jobs[jb].wfnc;
    const int ncols = wfnc.sh.nsec(1);
    for (size_t b = 0; b < wfnc.tags.size(); ++b) {
      const int i = static_cast<int>(wfnc.tags[b] / ncols), j = static_cast<int>(wfnc.tags[b] % ncols);
      const int m = wfnc.sh.dshape[0][i], n = wfnc.sh.dshape[1][j];
      if (m == 0 || n == 0) continue;
      const int k = std::min(m, n);
      Blk x{static_cast<int>(jb), wfnc.d + wfnc.offsets[b], static_cast<int32_t>(b), i, j, m, n, k, 0, 0, 0};
      x.s_off = nsv;
      nsv += k;
      maxmn = std::max<int64_t>(maxmn, int64_t(m) * n);
      blks.push_back(x);
    }
  }
  // Device layout (doubles): singular values | gesvd info per block (two ints per
  // double) | U and V^T per block.  The head (values and infos) is read back.
  const int64_t info_off = (nsv + 1) & ~int64_t(1);
  const int64_t head = info_off + (static_cast<int64_t>(blks.size()) + 1) / 2 + 1;
  int64_t tot = head;
  for (auto& x : blks) {
    x.u_off = tot;
    tot += int64_t(x.m) * x.k;
    x.v_off = tot;
    tot += int64_t(x.k) * x.n;
  }
  // Lanes take blocks largest first; each lane has its own workspace.
  ctx.svd_mats.ensure(size_t(tot) * sizeof(double), ctx.stream);
  double* mats = ctx.svd_mats.as<double>();
  int* infos = reinterpret_cast<int*>(mats + info_off);
  // statuses of blocks that write none (batched eigensolver route) read as success
  cuda_check(cudaMemsetAsync(infos, 0, size_t(head - info_off) * sizeof(double), ctx.stream), "svd info zero");
  // Blocks whose working copy fits in shared memory go to one launch of the batched
  // Jacobi SVD kernel.  Of the rest, blocks with min(m, n) >= kEighMin take the
  // reduced-density-matrix route: the eigenvectors of A A^T (forward) or A^T A
  // (backward) give the kept factor, the other one is a projection of A (cuSOLVER's
  // gesvd is latency-bound at these sizes); the others take gesvd.
  int lwork = 0;
  int64_t max_gram = 1;
  std::vector<DSvdBlock> jac;
  size_t jac_smem = 0;
  const int jac_cols = ctx.svd_jacobi_cols >= 0 ? std::min(ctx.svd_jacobi_cols, kJacobiMaxCols) : kJacobiUseCols;
  const int gram_max = ctx.svd_gram_max >= 0 ? ctx.svd_gram_max : kGramBatchMax;
  std::vector<int> gram;  // blocks of the batched eigensolver route
  std::map<int, int> per_p;  // candidates per padded Gram size
  auto gram_dim = [&](const Blk& x) { return jobs[x.job].forward ? x.m : x.n; };
  auto jac_ok = [&](const Blk& x, int cols) {
    return x.k <= cols && jacobi_svd_smem(x.m, x.n) <= kJacobiMaxSmem;
  };
  auto to_jacobi = [&](Blk& x, size_t bi) {
    x.jacobi = true;
    jac.push_back(DSvdBlock{x.a, x.u_off, x.s_off, x.v_off, x.m, x.n, static_cast<int>(bi), 0});
    jac_smem = std::max(jac_smem, jacobi_svd_smem(x.m, x.n));
  };
  // Default routing: blocks up to kJacobiFirstCols columns always take the Jacobi
  // kernel; larger ones take the batched eigensolver when their padded size is
  // shared by enough blocks, else the Jacobi kernel up to kJacobiUseCols columns (its
  // cost grows steeply with the columns), else the lanes.  Routing set by the caller
  // applies its limits as given.
  const bool by_default = ctx.svd_jacobi_cols < 0;
  const int first_cols = by_default ? std::min(kJacobiFirstCols, jac_cols) : jac_cols;
  for (size_t bi = 0; bi < blks.size(); ++bi) {
    Blk& x = blks[bi];
    if (jac_ok(x, first_cols))
      to_jacobi(x, bi);
    else if (gram_dim(x) <= gram_max)
      ++per_p[(gram_dim(x) + 7) & ~7];
  }
  // an explicit Gram limit (routing set by the caller) takes every candidate
  const int min_batch = ctx.svd_gram_max >= 0 ? 1 : kGramMinBatch;
  for (size_t bi = 0; bi < blks.size(); ++bi) {
    Blk& x = blks[bi];
    if (x.jacobi) continue;
    if (gram_dim(x) <= gram_max && per_p[(gram_dim(x) + 7) & ~7] >= min_batch) {
      x.gram = true;
      x.eigh = true;
      gram.push_back(static_cast<int>(bi));
    } else if (jac_ok(x, jac_cols)) {
      to_jacobi(x, bi);
    }
  }
  for (auto& x : blks) {
    if (x.jacobi || x.gram) continue;
    int lw = 0;
    x.eigh = x.k >= kEighMin;
    if (x.eigh) {
      const int d = jobs[x.job].forward ? x.m : x.n;
      solver_check(cusolverDnDsyevd_bufferSize(ctx.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d,
                                               nullptr, d, nullptr, &lw),
                   "syevd bufferSize");
      max_gram = std::max<int64_t>(max_gram, int64_t(d) * d + d);
    } else {
      solver_check(cusolverDnDgesvd_bufferSize(ctx.solver, std::max(x.m, x.n), std::min(x.m, x.n), &lw),
                   "gesvd bufferSize");
    }
    lwork = std::max(lwork, lw);
  }
  // per lane: solver work | rwork | col-major copy of A | col-major U | col-major V^T | Gram + eigenvalues
  const size_t lane_doubles = size_t(lwork) + 8 + 4 * size_t(std::max<int64_t>(maxmn, 1)) + 8 + size_t(max_gram);
  std::vector<int> by_cost;
  for (size_t bi = 0; bi < blks.size(); ++bi)
    if (!blks[bi].jacobi && !blks[bi].gram) by_cost.push_back(static_cast<int>(bi));
  std::stable_sort(by_cost.begin(), by_cost.end(), [&](int p, int q) {
    return double(blks[p].m) * blks[p].n * blks[p].k > double(blks[q].m) * blks[q].n * blks[q].k;
  });
  const int hw = std::max(1, static_cast<int>(std::thread::hardware_concurrency()));
  const int nlanes = std::min({kSvdLanes, hw, static_cast<int>(by_cost.size())});
  while (static_cast<int>(ctx.svd_lanes.size()) < nlanes) {
    auto l = std::make_unique<Context::SvdLane>();
    cuda_check(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking), "svd lane stream");
    cuda_check(cudaEventCreateWithFlags(&l->done, cudaEventDisableTiming), "svd lane event");
    solver_check(cusolverDnCreate(&l->solver), "cusolverDnCreate");
    solver_check(cusolverDnSetStream(l->solver, l->stream), "cusolverDnSetStream");
    if (cublasCreate(&l->blas) != CUBLAS_STATUS_SUCCESS || cublasSetStream(l->blas, l->stream) != CUBLAS_STATUS_SUCCESS)
      throw Error(kCuda, "cublas handle for the SVD lanes");
    register_cache_stream(l->stream);
    ctx.svd_lanes.push_back(std::move(l));
  }
  if (!ctx.svd_ready) cuda_check(cudaEventCreateWithFlags(&ctx.svd_ready, cudaEventDisableTiming), "svd event");
  cuda_check(cudaEventRecord(ctx.svd_ready, st), "svd ready");
  // the small blocks on the context's stream, concurrently with the lanes
  DevArray<DSvdBlock> djac;
  if (!jac.empty()) {
    // (with profiling on, each route is timed on its own: the sub-phases synchronise)
    PhaseTimer tj(ctx, kPhSvdJacobi);
    djac.upload(jac, st);
    launch_jacobi_svd(djac.get(), static_cast<int>(jac.size()), jac_smem, mats, infos, st);
    ctx.kernel_launches += 1;
    tj.stop();
    ctx.timers[kPhSvdSolve] -= tj.dt;
  }
  // The batched eigensolver route, also on the context's stream: the Gram matrices of
  // all its blocks in one grouped GEMM, padded to multiples of 8 (-1 on the padded
  // diagonal keeps the padding's eigenvectors apart, below every eigenvalue of a
  // Gram matrix of a normalised wavefunction), one batched symmetric eigensolver call
  // per padded size, the leading eigenvectors as the isometric factor, and the other
  // factor (carrying s) from one grouped projection GEMM.  Replaces one latency-bound
  // solver call per block.
  std::vector<int> gram_info(gram.size(), 0);
  DevArray<DEigBlock> deig;
  int* gram_info_d = nullptr;
  std::vector<char> gram_host_work;
  if (!gram.empty()) {
    PhaseTimer tg(ctx, kPhSvdGram);
    if (!ctx.blas) {
      if (cublasCreate(&ctx.blas) != CUBLAS_STATUS_SUCCESS || cublasSetStream(ctx.blas, st) != CUBLAS_STATUS_SUCCESS)
        throw Error(kCuda, "cublas handle for the batched eigensolver route");
    }
    if (!ctx.solver_params) solver_check(cusolverDnCreateParams(&ctx.solver_params), "cusolverDnCreateParams");
    std::map<int, std::vector<int>> by_p;  // padded size -> blocks
    for (int bi : gram) by_p[(gram_dim(blks[bi]) + 7) & ~7].push_back(bi);
    struct PGroup {
      int P, cnt, first;
      int64_t g0, w0;
    };
    std::vector<PGroup> pg;
    std::vector<int> order;
    int64_t gtot = 0;
    for (auto& kv : by_p) {
      const int P = kv.first, cnt = static_cast<int>(kv.second.size());
      pg.push_back(PGroup{P, cnt, static_cast<int>(order.size()), gtot, gtot + int64_t(cnt) * P * P});
      gtot += int64_t(cnt) * P * P + int64_t(cnt) * P;
      order.insert(order.end(), kv.second.begin(), kv.second.end());
    }
    const int64_t ginfo_off = gtot;
    gtot += (static_cast<int64_t>(order.size()) + 1) / 2 + 1;
    ctx.svd_gram.ensure(size_t(gtot) * sizeof(double), st);
    double* gb = ctx.svd_gram.as<double>();
    gram_info_d = reinterpret_cast<int*>(gb + ginfo_off);
    const int ng = static_cast<int>(order.size());
    std::vector<DEigBlock> eb(ng);
    std::vector<cublasOperation_t> ta1(ng), tb1(ng), ta2(ng), tb2(ng);
    std::vector<int> m1(ng), n1(ng), k1(ng), lda1(ng), ldb1(ng), ldc1(ng);
    std::vector<int> m2(ng), n2(ng), k2(ng), lda2(ng), ldb2(ng), ldc2(ng);
    std::vector<double> one(ng, 1.0), zero(ng, 0.0);
    std::vector<int> gsize(ng, 1);
    std::vector<const double*> ptrs(6 * size_t(ng));  // A1 | B1 | C1 | A2 | B2 | C2
    for (const PGroup& g : pg) {
      for (int i = 0; i < g.cnt; ++i) {
        const int pos = g.first + i;
        const Blk& x = blks[order[pos]];
        const bool fw = jobs[x.job].forward;
        const int d = fw ? x.m : x.n;
        const int64_t goff = g.g0 + int64_t(i) * g.P * g.P;
        eb[pos] = DEigBlock{gb + g.w0 + int64_t(i) * g.P, fw ? mats + x.u_off : mats + x.v_off, mats + x.s_off, goff,
                            g.P, d, x.k, fw ? 0 : 1};
        // Gram matrix (column-major view of the row-major block: n x m, ld n)
        ta1[pos] = fw ? CUBLAS_OP_T : CUBLAS_OP_N;
        tb1[pos] = fw ? CUBLAS_OP_N : CUBLAS_OP_T;
        m1[pos] = n1[pos] = d;
        k1[pos] = fw ? x.n : x.m;
        lda1[pos] = ldb1[pos] = x.n;
        ldc1[pos] = g.P;
        ptrs[pos] = x.a;
        ptrs[ng + pos] = x.a;
        ptrs[2 * size_t(ng) + pos] = gb + goff;
        // projection: forward s V^T = U^T A (k x n row-major = A^T U column-major);
        // backward U s = A V (m x k row-major = V^T A^T column-major)
        if (fw) {
          ta2[pos] = CUBLAS_OP_N;
          tb2[pos] = CUBLAS_OP_T;
          m2[pos] = x.n;
          n2[pos] = x.k;
          k2[pos] = x.m;
          lda2[pos] = x.n;
          ldb2[pos] = x.k;
          ldc2[pos] = x.n;
          ptrs[3 * size_t(ng) + pos] = x.a;
          ptrs[4 * size_t(ng) + pos] = mats + x.u_off;
          ptrs[5 * size_t(ng) + pos] = mats + x.v_off;
        } else {
          ta2[pos] = CUBLAS_OP_T;
          tb2[pos] = CUBLAS_OP_N;
          m2[pos] = x.k;
          n2[pos] = x.m;
          k2[pos] = x.n;
          lda2[pos] = x.n;
          ldb2[pos] = x.n;
          ldc2[pos] = x.k;
          ptrs[3 * size_t(ng) + pos] = mats + x.v_off;
          ptrs[4 * size_t(ng) + pos] = x.a;
          ptrs[5 * size_t(ng) + pos] = mats + x.u_off;
        }
      }
    }
    ctx.svd_ptrs.ensure(ptrs.size() * sizeof(double*), st);
    upload_staged(ctx.svd_ptrs.p, ptrs.data(), ptrs.size() * sizeof(double*), st);
    const double* const* dp = reinterpret_cast<const double* const*>(ctx.svd_ptrs.p);
    double* const* dc1 = reinterpret_cast<double* const*>(ctx.svd_ptrs.as<double*>() + 2 * size_t(ng));
    double* const* dc2 = reinterpret_cast<double* const*>(ctx.svd_ptrs.as<double*>() + 5 * size_t(ng));
    deig.upload(eb, st);
    cuda_check(cudaMemsetAsync(gb, 0, size_t(ginfo_off) * sizeof(double), st), "gram zero");
    launch_gram_pad(deig.get(), ng, gb, st);
    if (cublasDgemmGroupedBatched(ctx.blas, ta1.data(), tb1.data(), m1.data(), n1.data(), k1.data(), one.data(), dp,
                                  lda1.data(), dp + ng, ldb1.data(), zero.data(), dc1, ldc1.data(), ng,
                                  gsize.data()) != CUBLAS_STATUS_SUCCESS)
      throw Error(kCuda, "canonicalize: grouped Gram GEMM failed");
    size_t dev_bytes = 0, host_bytes = 0;
    for (const PGroup& g : pg) {
      size_t db = 0, hb = 0;
      solver_check(cusolverDnXsyevBatched_bufferSize(ctx.solver, ctx.solver_params, CUSOLVER_EIG_MODE_VECTOR,
                                                     CUBLAS_FILL_MODE_LOWER, g.P, CUDA_R_64F, gb + g.g0, g.P,
                                                     CUDA_R_64F, gb + g.w0, CUDA_R_64F, &db, &hb, g.cnt),
                   "syevBatched bufferSize");
      dev_bytes = std::max(dev_bytes, db);
      host_bytes = std::max(host_bytes, hb);
    }
    ctx.svd_gram_work.ensure(std::max<size_t>(dev_bytes, 16), st);
    gram_host_work.resize(std::max<size_t>(host_bytes, 16));
    for (const PGroup& g : pg)
      solver_check(cusolverDnXsyevBatched(ctx.solver, ctx.solver_params, CUSOLVER_EIG_MODE_VECTOR,
                                          CUBLAS_FILL_MODE_LOWER, g.P, CUDA_R_64F, gb + g.g0, g.P, CUDA_R_64F,
                                          gb + g.w0, CUDA_R_64F, ctx.svd_gram_work.p, dev_bytes,
                                          gram_host_work.data(), host_bytes, gram_info_d + g.first, g.cnt),
                   "syevBatched");
    launch_eig_factors_batched(deig.get(), ng, gb, st);
    if (cublasDgemmGroupedBatched(ctx.blas, ta2.data(), tb2.data(), m2.data(), n2.data(), k2.data(), one.data(),
                                  dp + 3 * size_t(ng), lda2.data(), dp + 4 * size_t(ng), ldb2.data(), zero.data(), dc2,
                                  ldc2.data(), ng, gsize.data()) != CUBLAS_STATUS_SUCCESS)
      throw Error(kCuda, "canonicalize: grouped projection GEMM failed");
    ctx.kernel_launches += 4 + static_cast<int64_t>(pg.size());
    tg.stop();
    ctx.timers[kPhSvdSolve] -= tg.dt;
  }
  std::atomic<int> next{0};
  std::vector<std::exception_ptr> errs(nlanes);
  std::vector<int64_t> lane_launches(nlanes, 0);
  auto lane_fn = [&](int li) {
    try {
      cuda_check(cudaSetDevice(ctx.device), "cudaSetDevice");
      Context::SvdLane& ln = *ctx.svd_lanes[li];
      cudaStream_t ls = ln.stream;
      cuda_check(cudaStreamWaitEvent(ls, ctx.svd_ready, 0), "svd lane wait");
      ln.work.ensure(lane_doubles * sizeof(double), ls);
      double* work = ln.work.as<double>();
      double* rwork = work + lwork + 8;
      double* tA = rwork + std::max<int64_t>(maxmn, 1);  // col-major working copy of the block
      double* tU = tA + maxmn;                           // col-major U when transposes are needed
      double* tV = tU + maxmn;                           // col-major VT when transposes are needed
      for (int i = next.fetch_add(1); i < static_cast<int>(by_cost.size()); i = next.fetch_add(1)) {
        const Blk& x = blks[by_cost[i]];
        const bool forward = jobs[x.job].forward;
        const double* a = x.a;
        double* U = mats + x.u_off;
        double* S = mats + x.s_off;
        double* V = mats + x.v_off;
        int* info = infos + by_cost[i];
        if (x.eigh) {
          double* G = tV + maxmn;
          const double one = 1.0, zero = 0.0;
          const int d = forward ? x.m : x.n;
          double* W = G + int64_t(d) * d;
          // a: row-major m x n == column-major n x m (ld n)
          cublasStatus_t bs =
              forward ? cublasDgemm(ln.blas, CUBLAS_OP_T, CUBLAS_OP_N, x.m, x.m, x.n, &one, a, x.n, a, x.n, &zero, G,
                                    x.m)
                      : cublasDgemm(ln.blas, CUBLAS_OP_N, CUBLAS_OP_T, x.n, x.n, x.m, &one, a, x.n, a, x.n, &zero, G,
                                    x.n);
          if (bs != CUBLAS_STATUS_SUCCESS) throw Error(kCuda, "canonicalize: Gram matrix dgemm failed");
          solver_check(cusolverDnDsyevd(ln.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, d, G, d, W, work,
                                        lwork, info),
                       "syevd");
          // forward: U (row-major m x k) and s V^T = U^T A; backward: V^T (row-major k x n) and U s = A V
          launch_eig_factors(G, W, d, x.k, forward ? 0 : 1, forward ? U : V, tU, S, ls);
          bs = forward ? cublasDgemm(ln.blas, CUBLAS_OP_N, CUBLAS_OP_N, x.n, x.k, x.m, &one, a, x.n, tU, x.m, &zero,
                                     V, x.n)
                       : cublasDgemm(ln.blas, CUBLAS_OP_T, CUBLAS_OP_N, x.k, x.m, x.n, &one, tU, x.n, a, x.n, &zero,
                                     U, x.k);
          if (bs != CUBLAS_STATUS_SUCCESS) throw Error(kCuda, "canonicalize: projection dgemm failed");
          lane_launches[li] += 1;
        } else if (x.n >= x.m) {
          // row-major A (m x n) is col-major A^T (n x m): A^T = Ux S VxT, so U_A = VxT buffer, Vt_A = Ux buffer
          cuda_check(cudaMemcpyAsync(tA, a, int64_t(x.m) * x.n * sizeof(double), cudaMemcpyDeviceToDevice, ls),
                     "svd copy");
          solver_check(cusolverDnDgesvd(ln.solver, 'S', 'S', x.n, x.m, tA, x.n, S, V, x.n, U, x.m, work, lwork,
                                        rwork, info),
                       "gesvd");
        } else {
          // col-major copy of A (m x n) = row-major A^T (n x m)
          launch_transpose(a, tA, x.m, x.n, ls);
          solver_check(cusolverDnDgesvd(ln.solver, 'S', 'S', x.m, x.n, tA, x.m, S, tU, x.m, tV, x.n, work, lwork,
                                        rwork, info),
                       "gesvd");
          // tU col-major (m x k) == row-major (k x m): transpose into row-major U (m x k)
          launch_transpose(tU, U, x.k, x.m, ls);
          // tV col-major (k x n) == row-major (n x k): transpose into row-major Vt (k x n)
          launch_transpose(tV, V, x.n, x.k, ls);
          lane_launches[li] += 3;
        }
      }
      cuda_check(cudaEventRecord(ln.done, ls), "svd lane done");
    } catch (...) {
      errs[li] = std::current_exception();
    }
  };
  {
    std::vector<std::thread> pool;
    for (int li = 1; li < nlanes; ++li) pool.emplace_back(lane_fn, li);
    if (nlanes > 0) lane_fn(0);
    for (auto& t : pool) t.join();
  }
  for (int li = 0; li < nlanes; ++li) {
    if (errs[li]) std::rethrow_exception(errs[li]);
    cuda_check(cudaStreamWaitEvent(st, ctx.svd_lanes[li]->done, 0), "svd join");
    ctx.kernel_launches += lane_launches[li];
  }
  // singular values and solver statuses to the host
  std::vector<double> hmats(head);
  cuda_check(cudaMemcpyAsync(hmats.data(), mats, head * sizeof(double), cudaMemcpyDeviceToHost, st), "s d2h");
  if (!gram.empty())
    cuda_check(cudaMemcpyAsync(gram_info.data(), gram_info_d, gram.size() * sizeof(int), cudaMemcpyDeviceToHost, st),
               "gram info d2h");
  ctx.sync();
  for (int v : gram_info)
    if (v != 0) throw Error(kSolver, "canonicalize: batched eigensolver did not converge (info " + std::to_string(v) + ")");
  {
    const int* hinfo = reinterpret_cast<const int*>(hmats.data() + info_off);
    for (size_t b = 0; b < blks.size(); ++b)
      if (hinfo[b] != 0)
        throw Error(kSolver, "canonicalize: block SVD did not converge (info " + std::to_string(hinfo[b]) + ")");
  }
  tsolve.stop();
  std::vector<CanonResult> results(jobs.size());
  for (size_t jb = 0; jb < jobs.size(); ++jb) {
  const bool forward = jobs[jb].forward;
  const DTensor& wfnc = *jobs[jb].wfnc;
  const int M = jobs[jb].M;
  PhaseTimer tselect(ctx, kPhSvdSelect);
  // sector of each block's singular values: row sector (LeftArrow) or column sector (RightArrow)
  std::map<int, size_t> sec_of;
  std::vector<std::vector<double>> svals;
  std::vector<int> secs;
  std::vector<int> blk_sv(blks.size());
  for (size_t b = 0; b < blks.size(); ++b) {
    if (blks[b].job != static_cast<int>(jb)) continue;
    const int sec = forward ? blks[b].i : blks[b].j;
    if (sec_of.count(sec)) throw Error(kInternal, "canonicalize: two blocks share one singular-value sector");
    sec_of[sec] = b;
  }
  for (auto& kv : sec_of) {
    const Blk& x = blks[kv.second];
    secs.push_back(kv.first);
    svals.emplace_back(hmats.begin() + x.s_off, hmats.begin() + x.s_off + x.k);
    blk_sv[kv.second] = static_cast<int>(svals.size() - 1);
  }
  CanonResult& res = results[jb];
  const double tie = ctx.tie_rtol >= 0.0 ? ctx.tie_rtol : kTieRtolDefault;
  std::vector<int> kept = select_kept(svals, M, tie, &res.discarded);
  // new bond sectors in ascending sector order
  std::vector<Qn> q_nz;
  std::vector<int> d_nz;
  std::map<int, int> newidx;
  for (size_t s = 0; s < secs.size(); ++s) {
    if (kept[s] <= 0) continue;
    const Qn qs = forward ? wfnc.sh.qshape[0][secs[s]] : -wfnc.sh.qshape[1][secs[s]];
    newidx[secs[s]] = static_cast<int>(q_nz.size());
    q_nz.push_back(qs);
    d_nz.push_back(kept[s]);
    res.kept.push_back({secs[s], kept[s]});
  }
  std::vector<Qn> neg_q_nz(q_nz.size());
  for (size_t s = 0; s < q_nz.size(); ++s) neg_q_nz[s] = -q_nz[s];
  auto U = std::make_unique<DTensor>();
  auto V = std::make_unique<DTensor>();
  U->sh.rank = 2;
  U->sh.q = forward ? Qn{} : wfnc.sh.q;
  U->sh.qshape = {wfnc.sh.qshape[0], neg_q_nz};
  U->sh.dshape = {wfnc.sh.dshape[0], d_nz};
  U->sh.finalize();
  V->sh.rank = 2;
  V->sh.q = forward ? wfnc.sh.q : Qn{};
  V->sh.qshape = {q_nz, wfnc.sh.qshape[1]};
  V->sh.dshape = {d_nz, wfnc.sh.dshape[1]};
  V->sh.finalize();
  struct Pl {
    int64_t ut, vt;
    size_t b;
  };
  std::vector<Pl> pl;
  for (size_t b = 0; b < blks.size(); ++b) {
    if (blks[b].job != static_cast<int>(jb)) continue;
    const int sec = forward ? blks[b].i : blks[b].j;
    auto it = newidx.find(sec);
    if (it == newidx.end()) continue;
    int ui[2] = {blks[b].i, it->second};
    int vi[2] = {it->second, blks[b].j};
    pl.push_back({U->sh.tag(ui), V->sh.tag(vi), b});
  }
  {
    std::vector<int64_t> ut, vt;
    for (auto& p : pl) {
      ut.push_back(p.ut);
      vt.push_back(p.vt);
    }
    std::sort(ut.begin(), ut.end());
    std::sort(vt.begin(), vt.end());
    U->set_blocks(ut);
    V->set_blocks(vt);
  }
  U->ctx = &ctx;
  V->ctx = &ctx;
  U->alloc_device(st, false);
  V->alloc_device(st, false);
  std::vector<DCopy> cu, cv;
  std::vector<double> s_kept;
  std::vector<int64_t> soff, boff;
  std::vector<int> brow, bcol;
  for (auto& p : pl) {
    const Blk& x = blks[p.b];
    const int k = kept[blk_sv[p.b]];
    const int32_t us = U->find(p.ut), vs = V->find(p.vt);
    cu.push_back(DCopy{U->offsets[us], x.u_off, x.m, k, k, x.k, 1.0});
    cv.push_back(DCopy{V->offsets[vs], x.v_off, k, x.n, x.n, x.n, 1.0});
    soff.push_back(static_cast<int64_t>(s_kept.size()));
    if (x.eigh)
      s_kept.insert(s_kept.end(), k, 1.0);  // the projected factor already carries s
    else
      s_kept.insert(s_kept.end(), hmats.begin() + x.s_off, hmats.begin() + x.s_off + k);
    if (forward) {
      boff.push_back(V->offsets[vs]);
      brow.push_back(k);
      bcol.push_back(x.n);
    } else {
      boff.push_back(U->offsets[us]);
      brow.push_back(x.m);
      bcol.push_back(k);
    }
  }
  tselect.stop();
  PhaseTimer tpost(ctx, kPhSvdPost);
  DevArray<DCopy> dcu, dcv;
  DevArray<double> ds;
  DevArray<int64_t> dso, dbo;
  DevArray<int> dbr, dbc;
  dcu.upload(cu, st);
  dcv.upload(cv, st);
  ds.upload(s_kept, st);
  dso.upload(soff, st);
  dbo.upload(boff, st);
  dbr.upload(brow, st);
  dbc.upload(bcol, st);
  launch_copy(dcu.get(), static_cast<int>(cu.size()), mats, U->d, 0, st);
  launch_copy(dcv.get(), static_cast<int>(cv.size()), mats, V->d, 0, st);
  if (forward)
    launch_scale_blocks_rows(V->d, dbo.get(), dbr.get(), dbc.get(), dso.get(), static_cast<int>(boff.size()),
                             ds.get(), st);
  else
    launch_scale_blocks_cols(U->d, dbo.get(), dbr.get(), dbc.get(), dso.get(), static_cast<int>(boff.size()),
                             ds.get(), st);
  ctx.kernel_launches += 3;
  res.lmat = std::move(U);
  res.rmat = std::move(V);
  }
  return results;
}

// ---------------------------------------------------------------------------
// make_noise (src/canonicalize.hpp:11-24)
// ---------------------------------------------------------------------------
// The reference builds the noise array as QSTArray(q, qshape, net dshape,
// bind(dist, rgen)).  STArray::generate and TArray::generate take the generator by
// value (include/btas/SPARSE/STArray.h:259-262, include/btas/DENSE/TArray.h:780-782),
// so every block is filled by its own copy of the freshly seeded engine: element j of
// any block (row-major) is the j-th value of one sequence, drawn here through the same
// standard-library engine and distribution.
std::vector<double> noise_sequence(int64_t n) {
  std::vector<double> seq(static_cast<size_t>(std::max<int64_t>(n, 0)));
  std::mt19937 rgen;
  std::uniform_real_distribution<double> dist(-1.0, 1.0);
  for (auto& v : seq) v = dist(rgen);
  return seq;
}

std::unique_ptr<DTensor> make_noise(Context& ctx, const DTensor& wfnc, double noise) {
  if (noise < 1.0e-8) return nullptr;
  const Shape& sh = wfnc.sh;
  // check_net_dshape (include/btas/SPARSE/STArray.h:386-401): the sector dimensions
  // seen in the stored blocks, 0 for sectors without one
  std::vector<std::vector<int>> net(sh.rank);
  for (int i = 0; i < sh.rank; ++i) net[i].assign(sh.nsec(i), 0);
  int idx[kMaxRank];
  for (int64_t t : wfnc.tags) {
    sh.index(t, idx);
    for (int i = 0; i < sh.rank; ++i) net[i][idx[i]] = sh.dshape[i][idx[i]];
  }
  // allocate() of the noise array (STArray.h:219-237): allowed blocks of non-zero
  // net size, ascending
  std::vector<int64_t> ntags;
  for (int64_t t = 0; t < sh.nsparse; ++t) {
    sh.index(t, idx);
    if (!sh.allowed(idx)) continue;
    int64_t n = 1;
    for (int i = 0; i < sh.rank; ++i) n *= net[i][idx[i]];
    if (n > 0) ntags.push_back(t);
  }
  // Axpy reserves the noise blocks wfnc lacks (include/btas/SPARSE/STBLAS.h:133-145)
  std::vector<int64_t> utags;
  std::set_union(wfnc.tags.begin(), wfnc.tags.end(), ntags.begin(), ntags.end(), std::back_inserter(utags));
  cudaStream_t st = ctx.stream;
  std::unique_ptr<DTensor> out = relayout(ctx, wfnc, utags);
  std::vector<DNoise> nb;
  int64_t nmax = 0;
  for (int64_t t : ntags) {
    const int32_t b = out->find(t);
    const int64_t n = out->block_size(b);
    nb.push_back(DNoise{out->offsets[b], n});
    nmax = std::max(nmax, n);
  }
  if (static_cast<int64_t>(ctx.noise_seq.n) < nmax) ctx.noise_seq.upload(noise_sequence(nmax), st);
  DevArray<DNoise> dnb;
  dnb.upload(nb, st);
  launch_noise_axpy(dnb.get(), static_cast<int>(nb.size()), ctx.noise_seq.get(), noise, out->d, st);
  ctx.kernel_launches += 1;
  return out;
}

CanonResult canonicalize(Context& ctx, bool forward, const DTensor& wfnc, int M, double noise) {
  std::unique_ptr<DTensor> noised = make_noise(ctx, wfnc, noise);
  std::vector<CanonResult> r = canonicalize_many(ctx, {CanonJob{forward, noised ? noised.get() : &wfnc, M}});
  if (noised) ctx.sync();  // the noised copy is freed on return
  return std::move(r[0]);
}

}  // namespace mpsxx
