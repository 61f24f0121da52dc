// Batched two-site steps: many independent bonds (the chains of a parameter scan)
// advanced together.  Their Davidson iterations run in lockstep: every
// H_eff * psi of all unconverged problems is one grouped tensor-core launch per
// stage (the problems' uneven quantum-number blocks in one persistent tile list),
// captured with its packing and split-K reduction as a CUDA graph, and the vector
// algebra is one batched launch per operation for all problems.  The algorithm per
// problem is the Davidson of src/diagonalize.hpp:310-449 with the split-precision
// refinement of the single-problem path.
#include <cmath>
#include <numeric>

#include "engine.hpp"
#include "jacobi.hpp"

namespace mpsxx {

namespace {

constexpr int kMaxRitz = 10;
constexpr int kSlotSigma = 10, kSlotRes = 20, kSlotDiag = 21, kSlotIn = 22, kSlotOut = 23, kSlots = 24;

struct Item {
  const DTensor *L, *R, *diag;
  DTensor* psi;
  SigmaPlan* sp;
  int64_t n = 0, off = 0;               // slice of the vector arena
  int64_t bL = 0, bR = 0, bPsi = 0, bScr = 0;  // byte bases in the packed arenas
  int64_t bL64 = 0, bR64 = 0, bScr64 = 0;       // element bases in the FP64 arenas
};

// One grouped FP64 H_eff * psi (slot kSlotIn -> kSlotOut of every member): the members'
// FP64 plans concatenated into one tile list per stage over the FP64 arenas.
struct Grouped64 {
  std::vector<int> members;
  DevArray<DTile> t1, t2;
  DevArray<DGemmTask> k1, k2;
  DevArray<DGemmPair> p1, p2;
  DevArray<DReduce> r1, r2;
  int n1 = 0, n2 = 0, nr1 = 0, nr2 = 0, slots = 0;
  Trans ta1 = kNoTrans, tb1 = kNoTrans, ta2 = kNoTrans, tb2 = kNoTrans;
};

// One grouped split-TF32 H_eff * psi: slot kSlotIn -> slot kSlotOut of every member.
struct Grouped {
  std::vector<int> members;
  DevArray<DBatchProb> probs;
  DevArray<DPack> packs;
  DevArray<DTile> t1, t2;
  DevArray<DGemmTask> k1, k2;
  DevArray<DPkPair> p1, p2;
  DevArray<DReduce> red;
  int npacks = 0, n1 = 0, n2 = 0, nred = 0, nslots = 0;
  int64_t nmax = 0;
  cudaGraphExec_t graph = nullptr;
  ~Grouped() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

class Batch {
 public:
  Batch(Context& ctx, std::vector<Item>& items) : ctx_(ctx), it_(items) {}

  void run_all(double tol, std::vector<DavidsonStats>& S, std::vector<double>& E) {
    const int N = static_cast<int>(it_.size());
    S.assign(N, DavidsonStats{});
    E.assign(N, 0.0);
    setup();
    std::vector<int> all(N);
    std::iota(all.begin(), all.end(), 0);
    if (ctx_.precision == kFP64) {
      davidson(all, tol, 0.0, 4, false, S, E);
    } else {
      davidson(all, tol, ctx_.split_floor, 4, false, S, E);
      for (int c = 0; c < N; ++c) S[c].energy_split = E[c];
      std::vector<int> todo = all;
      for (int round = 0; round < ctx_.refine_rounds && !todo.empty(); ++round) {
        std::vector<DavidsonStats> R(N);
        davidson(todo, tol, 0.0, 1, true, R, E);
        std::vector<int> next;
        for (int c : todo) {
          S[c].n_sigma += R[c].n_sigma;
          S[c].n_sigma_fp64 += R[c].n_sigma_fp64;
          S[c].micro += R[c].micro;
          S[c].macro += R[c].macro;
          S[c].rnorm = R[c].rnorm;
          S[c].rnorm_fp64 = R[c].rnorm_fp64;
          S[c].converged = R[c].converged;
          if (!R[c].converged) next.push_back(c);
        }
        todo.swap(next);
      }
    }
    check_device_error(ctx_);
    // Ritz vectors back into the wavefunctions, normalised
    upload_probs(all, all_probs_);
    launch_bproject(all_probs_.get(), N, nmax(all), vec_.as<double>(), 0, -1, part_.as<double>(), sums_.as<double>(),
                    ctx_.stream);
    for (int c = 0; c < N; ++c)
      cuda_check(cudaMemcpyAsync(it_[c].psi->d, vec_.as<double>() + it_[c].off, it_[c].n * sizeof(double),
                                 cudaMemcpyDeviceToDevice, ctx_.stream),
                 "batch result");
    ctx_.kernel_launches += 3;
    ctx_.sync();
  }

 private:
  Context& ctx_;
  std::vector<Item>& it_;
  DevBuf vec_, arL_, arR_, arPsi_, arScr_, part_, sums_, small_;
  DevBuf arL64_, arR64_, arScr64_;  // FP64 operators and stage-1 intermediates of all problems
  int64_t scr64_elems_ = 0;
  bool ar64_ready_ = false;
  std::unique_ptr<Grouped64> g64_;
  DevArray<DBatchProb> all_probs_, act_probs_;
  std::unique_ptr<Grouped> grp_;

  int64_t nmax(const std::vector<int>& s) const {
    int64_t m = 1;
    for (int c : s) m = std::max(m, it_[c].n);
    return m;
  }

  void upload_probs(const std::vector<int>& s, DevArray<DBatchProb>& out) {
    std::vector<DBatchProb> h;
    h.reserve(s.size());
    for (int c : s) h.push_back(DBatchProb{it_[c].off, it_[c].n});
    out.upload(h, ctx_.stream);
  }

  // arenas, initial vectors, diagonals and packed operators of every problem
  void setup() {
    const int N = static_cast<int>(it_.size());
    int64_t off = 0, bL = 0, bR = 0, bPsi = 0, bScr = 0;
    for (Item& x : it_) {
      x.n = x.psi->nnz;
      x.off = off;
      off += kSlots * std::max<int64_t>(x.n, 1);
      if (ctx_.precision != kFP64) {
        // one launch serves all members: their intermediates share the hi|lo format
        // (a plan tuned by a single-bond run may hold the FP32 one) and their L
        // operators the per-block layout (a single-bond plan may stack stage 1)
        if (x.sp->allow_stack) {
          x.sp->allow_stack = false;
          if (x.sp->stack1) x.sp->pk_built = false;
        }
        set_scr1_format(ctx_, *x.sp, *x.L, *x.R, false);
        x.bL = bL;
        bL += (x.sp->pk_L.bytes + 255) / 256 * 256;
        x.bR = bR;
        bR += (x.sp->pk_R.bytes + 255) / 256 * 256;
        x.bPsi = bPsi;
        bPsi += (x.sp->pk_psi.bytes + 255) / 256 * 256;
        x.bScr = bScr;
        bScr += (x.sp->pk_scr1.bytes + 255) / 256 * 256;
      }
    }
    vec_.ensure(size_t(std::max<int64_t>(off, 1)) * sizeof(double), ctx_.stream);
    cuda_check(cudaMemsetAsync(vec_.p, 0, size_t(std::max<int64_t>(off, 1)) * sizeof(double), ctx_.stream),
               "batch zero");
    part_.ensure(size_t(N) * kBatchBlocks * kMaxDot * kMaxDot * sizeof(double), ctx_.stream);
    sums_.ensure(size_t(N) * 2 * sizeof(double) + 64, ctx_.stream);
    small_.ensure(size_t(N) * (2 * kMaxDot * kMaxDot + 2) * sizeof(double), ctx_.stream);
    for (Item& x : it_) {
      double* base = vec_.as<double>() + x.off;
      cuda_check(cudaMemcpyAsync(base, x.psi->d, x.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx_.stream),
                 "batch psi");
      cuda_check(cudaMemcpyAsync(base + kSlotDiag * x.n, x.diag->d, x.n * sizeof(double), cudaMemcpyDeviceToDevice,
                                 ctx_.stream),
                 "batch diag");
    }
    if (ctx_.precision != kFP64) {
      arL_.ensure(std::max<int64_t>(bL, 16), ctx_.stream);
      arR_.ensure(std::max<int64_t>(bR, 16), ctx_.stream);
      arPsi_.ensure(std::max<int64_t>(bPsi, 16), ctx_.stream);
      arScr_.ensure(std::max<int64_t>(bScr, 16), ctx_.stream);
      for (Item& x : it_) {
        launch_pack(x.sp->pk_L.packs.get(), static_cast<int>(x.sp->pk_L.h_packs.size()), x.L->d,
                    arL_.as<uint8_t>() + x.bL, ctx_.stream);
        launch_pack(x.sp->pk_R.packs.get(), static_cast<int>(x.sp->pk_R.h_packs.size()), x.R->d,
                    arR_.as<uint8_t>() + x.bR, ctx_.stream);
        ctx_.kernel_launches += 2;
      }
    }
  }

  // FP64 arenas: every problem's merged operators copied side by side (once per batch)
  void setup_fp64() {
    int64_t nL = 0, nR = 0, nS = 0;
    for (Item& x : it_) {
      x.bL64 = nL;
      nL += (x.L->nnz + 31) / 32 * 32;
      x.bR64 = nR;
      nR += (x.R->nnz + 31) / 32 * 32;
      x.bScr64 = nS;
      nS += (x.sp->scr1.nnz + 31) / 32 * 32;
    }
    arL64_.ensure(size_t(std::max<int64_t>(nL, 1)) * sizeof(double), ctx_.stream);
    arR64_.ensure(size_t(std::max<int64_t>(nR, 1)) * sizeof(double), ctx_.stream);
    arScr64_.ensure(size_t(std::max<int64_t>(nS, 1)) * sizeof(double), ctx_.stream);
    scr64_elems_ = nS;
    for (Item& x : it_) {
      if (x.L->nnz)
        cuda_check(cudaMemcpyAsync(arL64_.as<double>() + x.bL64, x.L->d, x.L->nnz * sizeof(double),
                                   cudaMemcpyDeviceToDevice, ctx_.stream),
                   "batch L64");
      if (x.R->nnz)
        cuda_check(cudaMemcpyAsync(arR64_.as<double>() + x.bR64, x.R->d, x.R->nnz * sizeof(double),
                                   cudaMemcpyDeviceToDevice, ctx_.stream),
                   "batch R64");
    }
    ar64_ready_ = true;
  }

  void build_grouped64(const std::vector<int>& members) {
    auto g = std::make_unique<Grouped64>();
    g->members = members;
    std::vector<DTile> t1, t2;
    std::vector<DGemmTask> k1, k2;
    std::vector<DGemmPair> p1, p2;
    std::vector<DReduce> r1, r2;
    int slots = 0;
    // one problem's stage into the grouped lists: operand bases a0, b0 and result base
    // c0 (elements), task, pair and split-K slot numbers shifted past the earlier ones
    auto add = [&](const GemmPlan& s, int64_t a0, int64_t b0, int64_t c0, std::vector<DTile>& T,
                   std::vector<DGemmTask>& K, std::vector<DGemmPair>& P, std::vector<DReduce>& R) {
      const int tb = static_cast<int>(K.size()), pb = static_cast<int>(P.size());
      for (DGemmTask t : s.h_tasks) {
        t.c_off += c0;
        t.p0 += pb;
        t.p1 += pb;
        K.push_back(t);
      }
      for (DGemmPair q : s.h_pairs) {
        q.a_off += a0;
        q.b_off += b0;
        P.push_back(q);
      }
      for (DTile t : s.h_tiles) {
        t.task += tb;
        t.p0 += pb;
        t.p1 += pb;
        if (t.slot >= 0) t.slot += slots;
        T.push_back(t);
      }
      for (DReduce r : s.h_reduce) {
        r.task += tb;
        r.slot0 += slots;
        R.push_back(r);
      }
    };
    int slots1 = 0;
    for (int c : members) {
      const Item& x = it_[c];
      add(x.sp->s1, x.bL64, x.off + kSlotIn * x.n, x.bScr64, t1, k1, p1, r1);
      slots += x.sp->s1.nslots;
    }
    slots1 = slots;
    slots = 0;
    for (int c : members) {
      const Item& x = it_[c];
      add(x.sp->s2, x.bScr64, x.bR64, x.off + kSlotOut * x.n, t2, k2, p2, r2);
      slots += x.sp->s2.nslots;
    }
    g->slots = std::max(slots1, slots);
    const GemmPlan& s0 = it_[members[0]].sp->s1;
    const GemmPlan& q0 = it_[members[0]].sp->s2;
    g->ta1 = s0.ta;
    g->tb1 = s0.tb;
    g->ta2 = q0.ta;
    g->tb2 = q0.tb;
    for (int c : members)
      if (it_[c].sp->s1.ta != g->ta1 || it_[c].sp->s1.tb != g->tb1 || it_[c].sp->s2.ta != g->ta2 ||
          it_[c].sp->s2.tb != g->tb2)
        throw Error(kInternal, "batched FP64 sigma: stage transposes differ between problems");
    g->n1 = static_cast<int>(t1.size());
    g->n2 = static_cast<int>(t2.size());
    g->nr1 = static_cast<int>(r1.size());
    g->nr2 = static_cast<int>(r2.size());
    g->t1.upload(t1, ctx_.stream);
    g->t2.upload(t2, ctx_.stream);
    g->k1.upload(k1, ctx_.stream);
    g->k2.upload(k2, ctx_.stream);
    g->p1.upload(p1, ctx_.stream);
    g->p2.upload(p2, ctx_.stream);
    g->r1.upload(r1, ctx_.stream);
    g->r2.upload(r2, ctx_.stream);
    g64_ = std::move(g);
  }

  // FP64 H_eff * psi of every member in one launch per stage (outputs zeroed by the caller)
  void sigma64_grouped(const std::vector<int>& act) {
    if (!ar64_ready_) setup_fp64();
    if (!g64_ || g64_->members != act) {
      PhaseTimer tg(ctx_, kPhBatchGroup);
      build_grouped64(act);
    }
    const Grouped64& g = *g64_;
    const cudaStream_t st = ctx_.stream;
    if (scr64_elems_)
      cuda_check(cudaMemsetAsync(arScr64_.p, 0, size_t(scr64_elems_) * sizeof(double), st), "batch scr64 zero");
    ctx_.gemm_part.ensure(std::max<size_t>(size_t(g.slots) * kGemmTile * kGemmTile * sizeof(double), 16), st);
    double* part = ctx_.gemm_part.as<double>();
    double* V = vec_.as<double>();
    launch_gemm_f64(g.ta1, g.tb1, 1.0, arL64_.as<double>(), V, arScr64_.as<double>(), g.t1.get(), g.n1, g.k1.get(),
                    g.p1.get(), part, st);
    if (g.nr1) launch_gemm_reduce(g.r1.get(), g.nr1, g.k1.get(), 1.0, part, arScr64_.as<double>(), st);
    launch_gemm_f64(g.ta2, g.tb2, 1.0, arScr64_.as<double>(), arR64_.as<double>(), V, g.t2.get(), g.n2, g.k2.get(),
                    g.p2.get(), part, st);
    if (g.nr2) launch_gemm_reduce(g.r2.get(), g.nr2, g.k2.get(), 1.0, part, V, st);
    ctx_.kernel_launches += 3 + (g.nr1 > 0) + (g.nr2 > 0);
  }

  // the grouped launch lists of a member set, and its graph
  void build_grouped(const std::vector<int>& members) {
    auto g = std::make_unique<Grouped>();
    g->members = members;
    std::vector<DPack> packs;
    std::vector<DTile> t1, t2;
    std::vector<DGemmTask> k1, k2;
    std::vector<DPkPair> p1, p2;
    std::vector<DReduce> red;
    int nslots = 0;
    for (int c : members) {
      const Item& x = it_[c];
      const SigmaPlan& sp = *x.sp;
      for (DPack pk : sp.pk_psi.h_packs) {
        pk.src_off += x.off + kSlotIn * x.n;
        pk.dst_off += x.bPsi;
        packs.push_back(pk);
      }
      const int tb1 = static_cast<int>(k1.size()), pb1 = static_cast<int>(p1.size());
      for (DGemmTask t : sp.h_pk_tasks1) {
        t.c_off += x.bScr;
        t.p0 += pb1;
        t.p1 += pb1;
        k1.push_back(t);
      }
      for (DPkPair pr : sp.h_pk1) {
        pr.a_pk += x.bL;
        pr.b_pk += x.bPsi;
        p1.push_back(pr);
      }
      for (DTile t : sp.s1.h_tiles_tc) {
        if (t.slot >= 0) throw Error(kInternal, "batched sigma: stage 1 is not split along K");
        t.task += tb1;
        t.p0 += pb1;
        t.p1 += pb1;
        t1.push_back(t);
      }
      const int tb2 = static_cast<int>(k2.size()), pb2 = static_cast<int>(p2.size()), sb = nslots;
      for (DGemmTask t : sp.s2.h_tasks) {
        t.c_off += x.off + kSlotOut * x.n;
        t.p0 += pb2;
        t.p1 += pb2;
        k2.push_back(t);
      }
      for (DPkPair pr : sp.h_pk2) {
        pr.a_pk += x.bScr;
        pr.b_pk += x.bR;
        p2.push_back(pr);
      }
      for (DTile t : sp.s2.h_tiles_tc) {
        t.task += tb2;
        t.p0 += pb2;
        t.p1 += pb2;
        if (t.slot >= 0) t.slot += sb;
        t2.push_back(t);
      }
      for (DReduce r : sp.s2.h_reduce_tc) {
        r.task += tb2;
        r.slot0 += sb;
        red.push_back(r);
      }
      nslots += sp.s2.nslots_tc;
    }
    // one persistent tile list per stage, heaviest first
    auto by_work = [](std::vector<DTile>& tiles, const std::vector<DPkPair>& pairs) {
      std::vector<std::pair<int64_t, size_t>> w(tiles.size());
      for (size_t i = 0; i < tiles.size(); ++i) {
        int64_t k = 0;
        for (int q = tiles[i].p0; q < tiles[i].p1; ++q) k += pairs[q].nks;
        w[i] = {-k, i};
      }
      std::stable_sort(w.begin(), w.end());
      std::vector<DTile> out(tiles.size());
      for (size_t i = 0; i < w.size(); ++i) out[i] = tiles[w[i].second];
      tiles.swap(out);
    };
    by_work(t1, p1);
    by_work(t2, p2);
    g->npacks = static_cast<int>(packs.size());
    g->n1 = static_cast<int>(t1.size());
    g->n2 = static_cast<int>(t2.size());
    g->nred = static_cast<int>(red.size());
    g->nslots = nslots;
    g->nmax = nmax(members);
    g->packs.upload(packs, ctx_.stream);
    g->t1.upload(t1, ctx_.stream);
    g->t2.upload(t2, ctx_.stream);
    g->k1.upload(k1, ctx_.stream);
    g->k2.upload(k2, ctx_.stream);
    g->p1.upload(p1, ctx_.stream);
    g->p2.upload(p2, ctx_.stream);
    g->red.upload(red, ctx_.stream);
    upload_probs(members, g->probs);
    ctx_.gemm_part.ensure(std::max<size_t>(size_t(nslots) * kTcTileM * kTcTileN * sizeof(double), 16), ctx_.stream);
    int* err = device_err_flag(ctx_);
    // the members' intermediates share one format (set in setup)
    const bool single = it_[members[0]].sp->scr1_single;
    const SigmaPlan& p0 = *it_[members[0]].sp;
    for (int c : members)
      if (it_[c].sp->scr1_single != single || it_[c].sp->ops_single != p0.ops_single)
        throw Error(kInternal, "batched sigma: operand formats differ");
    // capture: zero the outputs, pack the inputs, both stages, the split-K sums
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamBeginCapture(ctx_.stream, cudaStreamCaptureModeThreadLocal), "batch capture");
    const int nm = static_cast<int>(members.size());
    launch_bzero(g->probs.get(), nm, g->nmax, vec_.as<double>(), kSlotOut, ctx_.stream);
    launch_pack(g->packs.get(), g->npacks, vec_.as<double>(), arPsi_.as<uint8_t>(), ctx_.stream);
    launch_gemm_pk(arL_.as<uint8_t>(), arPsi_.as<uint8_t>(), 1.0, nullptr, arScr_.as<uint8_t>(), g->t1.get(), g->n1,
                   g->k1.get(), g->p1.get(), nullptr, single ? kOutPackedSingle : kOutPackedSplit, p0.stage1_single(), err, ctx_.stream,
                   ctx_.device_timeout_ns);
    launch_gemm_pk(arScr_.as<uint8_t>(), arR_.as<uint8_t>(), 1.0, vec_.as<double>(), nullptr, g->t2.get(), g->n2,
                   g->k2.get(), g->p2.get(), ctx_.gemm_part.as<double>(), kOutFP64, p0.stage2_single(), err, ctx_.stream,
                   ctx_.device_timeout_ns);
    launch_gemm_pk_reduce(g->red.get(), g->nred, g->k2.get(), 1.0, ctx_.gemm_part.as<double>(), vec_.as<double>(),
                          ctx_.stream);
    cuda_check(cudaStreamEndCapture(ctx_.stream, &graph), "batch capture end");
    cudaError_t e = cudaGraphInstantiate(&g->graph, graph, 0);
    cudaGraphDestroy(graph);
    cuda_check(e, "batch graph instantiate");
    grp_ = std::move(g);
  }

  // sigma of trial slot k for the active problems (prec: FP64 per problem, or one
  // grouped split launch whose members cover the active set)
  void sigma(const std::vector<int>& act, int k, int prec, std::vector<DavidsonStats>& S) {
    PhaseTimer tm(ctx_, prec == kFP64 && ctx_.precision != kFP64 ? kPhSigmaFP64 : kPhSigma);
    const int na = static_cast<int>(act.size());
    const int64_t nm = nmax(act);
    launch_bcopy(act_probs_.get(), na, nm, vec_.as<double>(), k, kSlotIn, ctx_.stream);
    if (prec == kFP64) {
      launch_bzero(act_probs_.get(), na, nm, vec_.as<double>(), kSlotOut, ctx_.stream);
      sigma64_grouped(act);
      for (int c : act) S[c].n_sigma_fp64 += 1;
    } else {
      // rebuild the grouped lists only when the active set has shrunk well below them
      bool ok = grp_ != nullptr;
      if (ok) {
        size_t j = 0;
        for (int c : act) {
          while (j < grp_->members.size() && grp_->members[j] < c) ++j;
          if (j == grp_->members.size() || grp_->members[j] != c) {
            ok = false;
            break;
          }
        }
        if (ok && act.size() * 4 < grp_->members.size() * 3) ok = false;
      }
      if (!ok) {
        PhaseTimer tg(ctx_, kPhBatchGroup);
        build_grouped(act);
        tg.stop();
        ctx_.timers[tm.phase] -= tg.dt;
      }
      cuda_check(cudaGraphLaunch(grp_->graph, ctx_.stream), "batch graph launch");
      ctx_.kernel_launches += 5;
    }
    for (int c : act) {
      S[c].n_sigma += 1;
      ctx_.sigma_flops += it_[c].sp->flops;
      ctx_.sigma_calls += 1;
    }
    launch_bcopy(act_probs_.get(), na, nm, vec_.as<double>(), kSlotOut, kSlotSigma + k, ctx_.stream);
    ctx_.kernel_launches += 2;
    tm.stop();
    ctx_.timers[kPhDavidsonRest] -= tm.dt;  // H_eff * psi is not part of the rest
  }

  // Davidson over the problems in `set`, in lockstep; the loop of the single path
  void davidson(std::vector<int> act, double tol, double rel_floor, int max_macro, bool anchor,
                std::vector<DavidsonStats>& S, std::vector<double>& E) {
    double* V = vec_.as<double>();
    double* Hdev = small_.as<double>();
    double* Rdev = Hdev + act.size() * kMaxDot * kMaxDot;
    double* Edev = Rdev + act.size() * kMaxDot * kMaxDot;
    for (int c : act) {
      S[c].converged = 0;
    }
    int niter = 0;
    std::vector<double> h, rv, ev, rn;
    while (!act.empty() && niter < max_macro) {
      PhaseTimer trest(ctx_, kPhDavidsonRest);
      upload_probs(act, act_probs_);
      int na = static_cast<int>(act.size());
      launch_bproject(act_probs_.get(), na, nmax(act), V, 0, -1, part_.as<double>(), sums_.as<double>(),
                      ctx_.stream);
      ctx_.kernel_launches += 3;
      sigma(act, 0, anchor && niter == 0 ? kFP64 : ctx_.precision, S);
      for (int m = 1; m <= kMaxRitz && !act.empty(); ++m) {
        na = static_cast<int>(act.size());
        launch_bmultidot(act_probs_.get(), na, V, m, part_.as<double>(), Hdev, ctx_.stream);
        h.resize(size_t(na) * kMaxDot * kMaxDot);
        cuda_check(cudaMemcpyAsync(h.data(), Hdev, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream),
                   "batch heff");
        ctx_.sync();
        rv.assign(size_t(na) * kMaxDot * kMaxDot, 0.0);
        ev.assign(na, 0.0);
        for (int a = 0; a < na; ++a) {
          std::vector<double> heff(m * m), rval, rvec;
          const double* hs = h.data() + size_t(a) * kMaxDot * kMaxDot;
          for (int i = 0; i < m; ++i)
            for (int j = 0; j <= i; ++j) {
              heff[i * m + j] = hs[i * m + j];
              heff[j * m + i] = hs[i * m + j];
            }
          jacobi_eigh(m, heff, rval, rvec);
          ev[a] = rval[0];
          std::copy(rvec.begin(), rvec.end(), rv.begin() + size_t(a) * kMaxDot * kMaxDot);
          S[act[a]].micro += 1;
        }
        upload_staged(Rdev, rv.data(), rv.size() * sizeof(double), ctx_.stream);
        upload_staged(Edev, ev.data(), ev.size() * sizeof(double), ctx_.stream);
        launch_brotate(act_probs_.get(), na, nmax(act), V, m, Rdev, ctx_.stream);
        launch_bresidual(act_probs_.get(), na, V, Edev, part_.as<double>(), sums_.as<double>(), ctx_.stream);
        ctx_.kernel_launches += 3;
        rn.resize(na);
        cuda_check(cudaMemcpyAsync(rn.data(), sums_.p, na * sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream),
                   "batch rnorm");
        ctx_.sync();
        std::vector<int> still;
        for (int a = 0; a < na; ++a) {
          const int c = act[a];
          E[c] = ev[a];
          S[c].rnorm = rn[a];
          if (anchor && niter == 0 && m == 1) S[c].rnorm_fp64 = rn[a];
          if (rn[a] < tol || (rel_floor > 0.0 && rn[a] < rel_floor * rel_floor * ev[a] * ev[a]))
            S[c].converged = 1;
          else
            still.push_back(c);
        }
        if (still.empty()) {
          act.clear();
          break;
        }
        if (still.size() != act.size()) {
          // the survivors' eigenvalues in their new order
          std::vector<double> ev2;
          for (int c : still) ev2.push_back(E[c]);
          upload_staged(Edev, ev2.data(), ev2.size() * sizeof(double), ctx_.stream);
          act.swap(still);
          upload_probs(act, act_probs_);
        }
        if (m < kMaxRitz) {
          na = static_cast<int>(act.size());
          const int64_t nm = nmax(act);
          launch_bprecondition(act_probs_.get(), na, nm, V, Edev, ctx_.stream);
          for (int i = 0; i < m; ++i)
            launch_bproject(act_probs_.get(), na, nm, V, kSlotRes, i, part_.as<double>(), sums_.as<double>(),
                            ctx_.stream);
          launch_bproject(act_probs_.get(), na, nm, V, kSlotRes, -1, part_.as<double>(), sums_.as<double>(),
                          ctx_.stream);
          launch_bcopy(act_probs_.get(), na, nm, V, kSlotRes, m, ctx_.stream);
          ctx_.kernel_launches += 1 + 3 * (m + 1) + 1;
          sigma(act, m, ctx_.precision, S);
        }
      }
      for (int c : act) S[c].macro += 1;
      ++niter;
    }
  }
};

}  // namespace

std::vector<double> diagonalize_batch(Context& ctx, const std::vector<const DTensor*>& L,
                                      const std::vector<const DTensor*>& R, const std::vector<const DTensor*>& diag,
                                      const std::vector<DTensor*>& psi, double tol, std::vector<DavidsonStats>& stats) {
  const size_t N = psi.size();
  if (L.size() != N || R.size() != N || diag.size() != N) throw Error(kInvalidArgument, "batch: argument counts");
  {
    // keep the references below valid: empty the cache only if this batch's plans do
    // not fit beside it (they are usually built already, by the planning threads)
    size_t missing = 0;
    for (size_t c = 0; c < N; ++c)
      missing += ctx.sigma_plans.count(std::make_tuple(L[c]->layout_id, R[c]->layout_id, psi[c]->layout_id)) == 0;
    if (ctx.sigma_plans.size() + missing > ctx.max_plans) ctx.sigma_plans.clear();
  }
  std::vector<Item> items(N);
  for (size_t c = 0; c < N; ++c) {
    if (diag[c]->nnz != psi[c]->nnz) throw Error(kInvalidArgument, "batch: diag and wavefunction layouts differ");
    items[c].L = L[c];
    items[c].R = R[c];
    items[c].diag = diag[c];
    items[c].psi = psi[c];
    items[c].sp = &sigma_plan(ctx, *L[c], *R[c], *psi[c]);
  }
  std::vector<double> E;
  Batch b(ctx, items);
  b.run_all(tol, stats, E);
  return E;
}

std::vector<BondOut> optimize_twosite_merged_batch(Context& ctx, const std::vector<BondArgs>& args, double tole) {
  const size_t N = args.size();
  std::vector<BondOut> out(N);
  std::vector<std::unique_ptr<DTensor>> mL(N), mR(N), psi(N);
  std::vector<DTensor> diag(N);
  std::vector<WaveMerge> wm(N);
  // Every bond's host plans first, on planning threads (they depend on layouts only):
  // merged operators, wavefunction merge, H_eff * psi (with its packed-operand plan)
  // and diagonal.  The device work then follows bond by bond on the stream.
  std::vector<std::unique_ptr<WavePlan>> wp(N);
  {
    PhaseTimer tp(ctx, kPhBatchPlan);
    reserve_plans(ctx, N);
    parallel_plan(ctx, static_cast<int>(N), [&](int c) {
      const BondArgs& a = args[c];
      const Tensor& L = merge_plan(ctx, true, *a.lmpo, *a.lopr).layout;
      const Tensor& R = merge_plan(ctx, false, *a.rmpo, *a.ropr).layout;
      wm[c] = wave_merge_infos(*a.lmpo, *a.rmpo, *a.lopr, *a.ropr);
      wp[c] = plan_merge_wave(ctx, wm[c], *a.lwfn, *a.rwfn);
      SigmaPlan& sp = sigma_plan(ctx, L, R, wp[c]->psi);
      diag_plan(ctx, L, R, wp[c]->psi);
      if (ctx.precision != kFP64) ensure_sigma_pk(ctx, sp, L, R);
    });
  }
  for (size_t c = 0; c < N; ++c) {
    const BondArgs& a = args[c];
    mL[c] = compute_merged_operator(ctx, true, *a.lmpo, *a.lopr);
    mR[c] = compute_merged_operator(ctx, false, *a.rmpo, *a.ropr);
    {
      PhaseTimer tw(ctx, kPhWaveMerge);
      psi[c] = run_merge_wave(ctx, *wp[c], *a.lwfn, *a.rwfn);
    }
    static_cast<Tensor&>(diag[c]) = static_cast<const Tensor&>(*psi[c]);
    diag[c].d = nullptr;
    diag[c].ctx = &ctx;
    diag[c].alloc_device(ctx.stream, true);
    compute_diagonal_elements(ctx, *mL[c], *mR[c], diag[c]);
  }
  std::vector<const DTensor*> Lp(N), Rp(N), Dp(N);
  std::vector<DTensor*> Pp(N);
  for (size_t c = 0; c < N; ++c) {
    Lp[c] = mL[c].get();
    Rp[c] = mR[c].get();
    Dp[c] = &diag[c];
    Pp[c] = psi[c].get();
  }
  std::vector<DavidsonStats> st;
  const std::vector<double> E = diagonalize_batch(ctx, Lp, Rp, Dp, Pp, tole, st);
  // all bonds' SVDs in one solve
  std::vector<CanonJob> jobs(N);
  std::vector<std::unique_ptr<DTensor>> noised(N);
  for (size_t c = 0; c < N; ++c) {
    noised[c] = make_noise(ctx, *psi[c], args[c].noise);
    jobs[c] = CanonJob{args[c].forward, noised[c] ? noised[c].get() : psi[c].get(), args[c].M};
  }
  std::vector<CanonResult> canon = canonicalize_many(ctx, jobs);
  {
    PhaseTimer tp(ctx, kPhBatchPlan);
    reserve_plans(ctx, N);
    parallel_plan(ctx, static_cast<int>(N), [&](int c) {
      const CanonResult& cr = canon[c];
      if (args[c].forward)
        renorm_plan(ctx, true, *mL[c], *cr.lmat, *cr.lmat);
      else
        renorm_plan(ctx, false, *mR[c], *cr.rmat, *cr.rmat);
    });
  }
  for (size_t c = 0; c < N; ++c) {
    const BondArgs& a = args[c];
    out[c].stats.energy = E[c];
    out[c].stats.dav = st[c];
    CanonResult& cr = canon[c];
    if (a.forward)
      out[c].env = renormalize(ctx, true, *mL[c], *cr.lmat, *cr.lmat);
    else
      out[c].env = renormalize(ctx, false, *mR[c], *cr.rmat, *cr.rmat);
    out[c].lwfn = expand_rows(ctx, wm[c].ql, *cr.lmat);
    out[c].rwfn = expand_cols(ctx, *cr.rmat, wm[c].qr);
  }
  release_bond_buffers(ctx);
  ctx.sync();
  return out;
}

}  // namespace mpsxx
