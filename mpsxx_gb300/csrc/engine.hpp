// Device engine of the merged two-site DMRG hot path.
#pragma once

#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <functional>
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <vector>

#include "kernels.hpp"
#include "qsd.hpp"

namespace mpsxx {

void cuda_check(cudaError_t e, const char* what);
void solver_check(cusolverStatus_t s, const char* what);
// the block cache serves a new stream (its blocks then wait on events when taken by
// another stream)
void register_cache_stream(cudaStream_t st);

// Grow-only device buffer.  Storage comes from the process-wide block cache:
// released blocks are kept for reuse instead of being returned with cudaFree, which
// would synchronise the device.  A buffer is used on the stream it was allocated on;
// its release records an event there, and a later owner on another stream waits for
// that event on the GPU before touching the block.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaStream_t st = nullptr;
  void ensure(size_t bytes, cudaStream_t stream);
  void release();
  ~DevBuf() { release(); }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

template <class T>
struct DevArray {
  DevBuf buf;
  size_t n = 0;
  void upload(const std::vector<T>& h, cudaStream_t st);  // allocates on st
  T* get() const { return buf.as<T>(); }
};

struct Context;

// Queued host-to-device copy of a small host array through pinned staging memory (the
// source may be reused as soon as the call returns).
void upload_staged(void* dst, const void* src, size_t bytes, cudaStream_t st);
// Drops a stream (drained, about to be destroyed) from the staging bookkeeping.
void forget_stream_uploads(cudaStream_t st);

// Lower roots projected out of the Davidson operator (multi-root targeting): device
// vectors in the wavefunction's layout and the roots' energies (at most 12).
constexpr size_t kMaxProjected = 12;
struct Projection {
  std::vector<const double*> S, H;
  std::vector<double> E;
};

// Device tensor: host layout descriptor + device storage (+ optional host data).
struct DTensor : Tensor {
  Context* ctx = nullptr;
  DevBuf store;
  std::vector<double> host;  // host copy for MPO coefficients (optional)
  void alloc_device(cudaStream_t st, bool zero = true);
};

// Grouped block GEMM plan built from the reference's task enumeration.
struct GemmPlan {
  Trans ta = kNoTrans, tb = kNoTrans;
  int K = 0;
  std::vector<GemmTaskRef> tasks;
  std::vector<DTile> h_tiles;
  std::vector<DGemmTask> h_tasks;
  std::vector<DGemmPair> h_pairs;
  std::vector<int32_t> pair_a_slot, pair_b_slot;  // operand block slots of h_pairs
  std::vector<int64_t> task_ctag;                 // result block tag of each h_tasks entry
  std::vector<DReduce> h_reduce;
  DevArray<DTile> tiles;
  DevArray<DGemmTask> dtasks;
  DevArray<DGemmPair> pairs;
  DevArray<DReduce> reduce;
  int nslots = 0;  // split-K partial tiles
  // tensor-core (split TF32) tiling of the same tasks: 128 x 128 tiles (64-row and
  // 64-column tails flagged per tile)
  std::vector<DTile> h_tiles_tc;
  std::vector<DReduce> h_reduce_tc;
  DevArray<DTile> tiles_tc;
  DevArray<DReduce> reduce_tc;
  int nslots_tc = 0;
  double flops = 0.0;
  int64_t c_elems = 0;  // elements of C touched (for traffic accounting)
  void upload(cudaStream_t st);
  // partial: nslots * 64 * 64 doubles of scratch (may be null when nslots == 0)
  void run(double alpha, const double* A, const double* B, double* C, double* partial, cudaStream_t st) const;
  size_t partial_bytes() const { return size_t(nslots) * kGemmTile * kGemmTile * sizeof(double); }
  size_t partial_bytes_tc() const { return size_t(nslots_tc) * kTcTileM * kTcTileN * sizeof(double); }
};

// Precision of the bulk contractions: kSplitTF32 runs H_eff * psi on the tensor
// cores, kSplitTF32All also the renormalisation contractions.
enum Precision : int { kFP64 = 0, kSplitTF32 = 1, kSplitTF32All = 2 };

// target number of CTAs a grouped GEMM is split into (a few waves on 152 SMs)
constexpr int kTargetCtas = 152 * 8;
// packed L*psi intermediates above this size make the tuner try w-blocked schedules
constexpr int64_t kGroupIntermediateBytes = int64_t(8) << 30;

// plans kept per kind in a context before the cache is emptied
constexpr size_t kMaxCachedPlans = 512;  // default of Context::max_plans
// Relative resolution of the split-TF32 operator: |H_split psi - H psi| stays below
// ~1e-5 |H psi| (measured a few 1e-6), so a residual under (1e-5 E)^2 is as converged
// as that operator allows.
constexpr double kSplitResidualFloorDefault = 1.0e-5;
// FP64-anchored refinement rounds of a split-precision diagonalisation
constexpr int kRefineRoundsDefault = 2;

// GEMM plan into a C whose layout is `c` (block offsets).  C blocks may be
// sub-blocks of a larger block when `cmap` is provided (fused merges).
void build_gemm_plan(GemmPlan& plan, Trans ta, Trans tb, const Tensor& a, const Tensor& b, const Tensor& c,
                     int K, std::vector<GemmTaskRef>&& tasks);

// Blocks of one tensor packed as split-TF32 tensor-core tiles (one role: A or B).
struct Packed {
  DevBuf buf;
  std::vector<int64_t> base;  // per block slot: byte offset of its tile grid (-1: not packed)
  std::vector<int> nks;       // per block slot: K slices
  std::vector<DPack> h_packs;
  DevArray<DPack> packs;
  int64_t bytes = 0;
  uint64_t src_layout = 0, src_version = ~0ull;  // what the buffer currently holds
};

// Split-TF32 execution of one GemmPlan: the operand blocks the plan touches are
// packed as tensor-core tiles from their FP64 storage, and the persistent kernel
// accumulates into the FP64 result (split-K partials reduced in a fixed order).
struct SplitGemm {
  Packed pa, pb;
  std::vector<DPkPair> h_pk;
  DevArray<DPkPair> pk;
};

struct SigmaPlan {
  std::mutex pk_mu;  // guards the packed-operand plan (built once, possibly by a planning thread)
  uint64_t l_id = 0, r_id = 0, psi_id = 0;
  Tensor scr1;  // layout of L*psi
  GemmPlan s1, s2;
  double flops = 0.0;
  int64_t bytes_min = 0;  // 8*(nnz L + nnz R + 2 nnz psi)
  // split-TF32 path over packed operands
  Tensor psi_layout;  // the wavefunction layout the plan was built for
  bool pk_built = false;
  // L*psi intermediate stored as FP32 tiles split on chip (true) or as hi|lo tiles:
  // half the HBM bytes against more shared-memory traffic; chosen by the autotuner
  bool scr1_single = false;
  // L and R packed as FP32 tiles split on chip (true) or as hi|lo tiles: half the
  // operators' HBM bytes; fixed when the plan is made (Context::sigma_fp32_operators)
  bool ops_single = false;
  // operand formats of the two stages' tensor-core launches (kSingleA / kSingleB)
  int stage1_single() const { return ops_single ? kSingleA : 0; }
  int stage2_single() const { return (scr1_single ? kSingleA : 0) | (ops_single ? kSingleB : 0); }
  Packed pk_L, pk_R, pk_psi, pk_scr1;
  // Stage 1 over stacked panels: the L blocks that multiply the same psi block (same
  // K and output columns) stacked row-wise into one operand, so that the ~70-row sector
  // blocks fill 128-row tiles.  pk_L then holds the panels; st1 tiles (task = a block of
  // the panel, p0 = panel), stpk1 one pair per panel (pad = its first row_map entry),
  // row_map the output block and row of every panel row.  Off for batched steps and
  // w-blocked schedules, which use the per-block layout.
  bool allow_stack = true;
  bool stack1 = false;
  std::vector<DTile> h_st1;
  std::vector<DPkPair> h_stpk1;
  std::vector<int64_t> h_row_map;
  DevArray<DTile> st1;
  DevArray<DPkPair> stpk1;
  DevArray<int64_t> row_map;
  std::vector<DPkPair> h_pk1, h_pk2;
  std::vector<DGemmTask> h_pk_tasks1;
  DevArray<DPkPair> pk1, pk2;
  DevArray<DGemmTask> pk_tasks1;
  // w-blocked execution: the MPO index w is cut into groups whose packed L*psi
  // intermediates fit a scratch of group_budget bytes; each group runs stage 1 then
  // stage 2 out of that scratch, which stays in L2 instead of going to HBM and back
  struct Group {
    int t1_begin = 0, t1_count = 0;  // stage-1 tiles (gt1)
    int t2_begin = 0, t2_count = 0;  // stage-2 tiles (gt2)
    int r_begin = 0, r_count = 0;    // split-K reductions (gred)
    int nslots = 0;
  };
  int64_t group_budget = -1;  // < 0: not tuned yet; 0: one pass over all of w (no groups)
  std::vector<Group> groups;
  int64_t group_scr_bytes = 0;
  int group_slots = 0;
  DevArray<DTile> gt1, gt2;
  DevArray<DGemmTask> gtasks1;  // stage-1 tasks with group-local packed output bases
  DevArray<DPkPair> gpk2;       // stage-2 pairs with group-local L*psi bases
  DevArray<DReduce> gred;
  DevBuf group_scr;
  double tuned_ms = 0.0;        // sigma time of the chosen budget when it was tuned
  // the grouped launch sequence captured as one CUDA graph, writing into `staged`;
  // valid while the buffers it was captured with stay where they are
  cudaGraphExec_t graph = nullptr;
  DevBuf staged;
  std::vector<const void*> graph_ptrs;
  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_ptrs.clear();
  }
  ~SigmaPlan() { drop_graph(); }
};

// Merged-operator scatter plan (result layout + destination/source records).
struct MergePlan {
  Tensor layout;
  DevArray<DScatterDst> dst;
  DevArray<DScatterSrc> src;
  int ndst = 0;
  // adjoint (MPO gradient): host copies of the destinations (pad = result block
  // slot), the MPO block of every source, and the sources grouped by MPO block
  std::vector<DScatterDst> h_dst;
  std::vector<int32_t> src_entry;
  int nentries = 0;
  bool adj_built = false;
  DevArray<int> adj_ptr, adj_idx;
};

// Renormalisation plan: both Gemm stages and the layouts they produce.
struct RenormPlan {
  Tensor scr, out;
  GemmPlan p1, p2;
  bool split_built = false;
  SplitGemm g1, g2;
};

struct DiagPlan {
  int max_tiles = 0;  // most 32 x 32 tiles of one block (the kernel's grid height)
  std::vector<DDiagTask> h_tasks;
  std::vector<DDiagPair> h_pairs;
  DevArray<DDiagTask> tasks;
  DevArray<DDiagPair> pairs;
  std::vector<std::pair<int64_t, std::vector<std::pair<int64_t, int64_t>>>> ref;  // (psi tag, [(L tag, R tag)])
};

// A two-site wavefunction merge: the merged layout and the grouped GEMM producing it.
struct WavePlan {
  Tensor psi;
  GemmPlan plan;
};

struct DavidsonStats {
  int n_sigma = 0;
  int macro = 0;
  int micro = 0;
  double rnorm = 0.0;
  int converged = 0;
  int n_sigma_fp64 = 0;       // applications in FP64 (all of them in FP64 precision)
  double energy_split = 0.0;  // Ritz value before refinement (split precision)
  double rnorm_fp64 = 0.0;    // |H psi - E psi|^2 with the FP64 operator (split precision)
};

// Phases of one bond step timed by Context::timers.
enum Phase {
  kPhMergePlan = 0,   // merged operators: host plan
  kPhMergeAlloc,      // merged operators: device allocation
  kPhMergeRun,        // merged operators: plan upload + scatter kernel
  kPhWaveMerge,       // two-site wavefunction merge
  kPhSigmaPlan,       // sigma / diagonal plans (host) and operand packing
  kPhSigma,           // H_eff * psi applications
  kPhDavidsonRest,    // Davidson without H_eff * psi
  kPhSvdSolve,        // per-block SVDs
  kPhSvdSelect,       // truncation and result layout (host)
  kPhSvdPost,         // U / sV^T copies and scaling
  kPhRenormPlan,      // renormalisation plans (host)
  kPhRenormRun,       // renormalisation contractions
  kPhSigmaFP64,       // FP64 H_eff * psi of the split path (refinement anchors)
  kPhBatchGroup,      // batched steps: grouped sigma lists and their graph capture
  kPhBatchPlan,       // batched steps: every bond's host plans (planning threads)
  kPhSvdJacobi,       // canonicalize: batched Jacobi kernel (part of svd_solve)
  kPhSvdGram,         // canonicalize: batched eigensolver route (part of svd_solve)
  kNumPhases
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cusolverDnHandle_t solver = nullptr;
  cusolverDnParams_t solver_params = nullptr;  // 64-bit solver API (batched eigensolver)
  cublasHandle_t blas = nullptr;               // on `stream` (grouped Gram/projection GEMMs)
  DevBuf svd_gram;   // Gram matrices, eigenvalues and infos of the batched eigensolver route
  DevBuf svd_gram_work;
  DevBuf svd_ptrs;   // device pointer arrays of the grouped GEMMs
  DevBuf scr1;       // sigma stage-1 intermediates
  DevBuf scr2;       // renormalize intermediates
  DevBuf work;       // Davidson vectors
  DevBuf partial;    // reduction partials
  DevBuf scalars;    // small device scalars
  DevBuf svd_work;   // solver workspace
  DevBuf svd_mats;   // per-block SVD matrices
  DevBuf gemm_part;  // split-K partial tiles
  DevBuf err_flag;   // device error flag of the tensor-core kernels
  // canonicalize: independent per-block SVDs run on these lanes concurrently, each
  // driven by its own host thread (the solver's launches are host-bound)
  struct SvdLane {
    cusolverDnHandle_t solver = nullptr;
    cublasHandle_t blas = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf work;
  };
  std::vector<std::unique_ptr<SvdLane>> svd_lanes;
  cudaEvent_t svd_ready = nullptr;
  int precision = kFP64;
  const Projection* projection = nullptr;  // set around a projected diagonalize
  // truncation: singular values within this relative window of the cutoff count as
  // equal to it and are kept together; < 0 selects the default (1e-10)
  double tie_rtol = -1.0;
  // split-precision sigma schedule chosen by the caller instead of the autotuner:
  // w scratch budget in bytes (0 = all of w at once) and stage-2 tile target; a
  // negative budget leaves the choice to the autotuner
  int64_t sigma_w_budget = -1;
  int sigma_target_tiles = 0;
  bool sigma_fp32_intermediate = false;  // with a forced schedule: FP32 L*psi tiles
  // split-precision H_eff*psi: merged operators packed as FP32 tiles (split into hi|lo
  // on chip: half the packed bytes, but the on-chip split of both operands makes the
  // kernel slower, 1.93 vs 1.56 ms at the C2 middle bond) instead of hi|lo TF32 tiles;
  // applies to plans made afterwards
  bool sigma_fp32_operators = false;
  uint64_t device_timeout_ns = kPkTimeoutNs;  // wait limit of the tensor-core kernels
  // canonicalize routing: blocks with min(m, n) <= svd_jacobi_cols go to the batched
  // Jacobi kernel, the rest with a Gram dimension <= svd_gram_max to the batched
  // eigensolver; < 0 selects the defaults
  int svd_jacobi_cols = -1;
  int svd_gram_max = -1;
  // split-precision diagonalize: the tensor-core Davidson stops at |r|^2 <
  // (split_floor * E)^2 (the operator's resolution); then up to refine_rounds
  // FP64-anchored continuations bring |r|^2 under the tolerance
  double split_floor = kSplitResidualFloorDefault;
  int refine_rounds = kRefineRoundsDefault;
  // make_noise: the leading values of the noise sequence on the device (grown on demand)
  DevArray<double> noise_seq;
  // plan caches are shared with the planning threads of a batched step: lookups and
  // insertions under plan_mu; while planning_threads is set no cache is emptied
  std::mutex plan_mu;
  bool planning_threads = false;
  // plans kept per kind before a cache is emptied (a batched scan of many chains
  // raises it so that converged sweeps find the previous sweep's plans)
  size_t max_plans = kMaxCachedPlans;
  std::map<std::tuple<uint64_t, uint64_t, uint64_t>, std::unique_ptr<SigmaPlan>> sigma_plans;
  std::map<std::tuple<uint64_t, uint64_t, uint64_t>, std::unique_ptr<DiagPlan>> diag_plans;
  std::map<std::tuple<int, uint64_t, uint64_t, uint64_t>, std::unique_ptr<MergePlan>> merge_plans;
  std::map<std::tuple<int, uint64_t, uint64_t, uint64_t>, std::unique_ptr<RenormPlan>> renorm_plans;
  // counters for measurement
  int64_t kernel_launches = 0;
  double sigma_flops = 0.0;
  int64_t sigma_calls = 0;
  // phase timers in seconds (enum Phase); accumulated only while profile is on,
  // each phase closing with a stream synchronisation
  bool profile = false;
  double timers[kNumPhases] = {};
  // last autotuning of a sigma plan: (scratch budget in bytes, milliseconds) pairs
  std::vector<double> last_tuning;

  explicit Context(int dev, cudaStream_t st);
  ~Context();
  void sync();
};

// Accumulates the time to its destruction (or stop()) into ctx.timers[phase] when
// profiling is on; the stream is synchronised first so device work is included.
struct PhaseTimer {
  Context& ctx;
  int phase;
  double t0 = 0.0;
  double dt = 0.0;  // measured duration (0 when profiling is off)
  bool open = true;
  bool on = false;  // profiling on and not on a planning thread
  PhaseTimer(Context& c, int ph);
  void stop();
  ~PhaseTimer() { stop(); }
};

// Packed-operand layouts of a sigma plan (built once), and one H_eff*psi of the plan
// in the given precision (sigma += H psi) — the building blocks of batched steps.
void ensure_sigma_pk(Context& ctx, SigmaPlan& p, const Tensor& L, const Tensor& R);
// the plan's L*psi intermediate as FP32 tiles split on chip (single) or hi|lo tiles
void set_scr1_format(Context& ctx, SigmaPlan& p, const Tensor& L, const Tensor& R, bool single);
void apply_sigma(Context& ctx, SigmaPlan& p, const DTensor& L, const DTensor& R, const double* psi, double* sigma,
                 int precision);

// Adjoint of compute_merged_operator: dE/dW for the MPO blocks given
// Y = dE/d(merged operator); and both site gradients of one bond's energy.
std::vector<double> mpo_gradient(Context& ctx, bool forward, const DTensor& mpo, const DTensor& opr,
                                 const DTensor& Y);
void bond_mpo_gradient(Context& ctx, const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr,
                       const DTensor& ropr, const DTensor& psi, std::vector<double>& gl, std::vector<double>& gr);

// Hand the packed-operand buffers of the cached plans back to the block cache.
void release_bond_buffers(Context& ctx);

// --- hot-path operations (reference names) ---------------------------------

// src/compute_sigma_vector.hpp:85-96: sigma += L psi R^T over (w, B').
SigmaPlan& sigma_plan(Context& ctx, const Tensor& L, const Tensor& R, const Tensor& psi);
void compute_sigma_vector(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& psi, DTensor& sigma);

int* device_err_flag(Context& ctx);
void check_device_error(Context& ctx);

// average device seconds of `reps` sigma applications (CUDA events on ctx.stream)
double sigma_device_time(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& psi, DTensor& sigma,
                         int reps);

// src/compute_diagonal_elements.hpp:65-80
DiagPlan& diag_plan(Context& ctx, const Tensor& L, const Tensor& R, const Tensor& diag);
// Work and bytes of a split-precision H_eff * psi plan: useful FLOPs of both stages,
// tensor-core tile FLOPs (tiles padded to 128 x 128 or their 64 tails, K slices of 32), K slices, tiles,
// packed bytes of L, R, the L*psi intermediate and psi, and the intermediate's size.
std::vector<double> sigma_plan_stats(Context& ctx, const Tensor& L, const Tensor& R, const Tensor& psi);
// Plans by layout (no device data read): cached, safe on planning threads.
const MergePlan& merge_plan(Context& ctx, bool forward, const DTensor& mpo, const Tensor& opr);
RenormPlan& renorm_plan(Context& ctx, bool forward, const Tensor& opr0, const Tensor& bra, const Tensor& ket);
// f(0..n-1) on up to 16 host threads with ctx.planning_threads set (plan building
// only: no launches); the first exception is rethrown after all threads joined
void parallel_plan(Context& ctx, int n, const std::function<void(int)>& f);
// empties the plan caches that could not take n more plans (call with no plan
// references held, before planning threads start)
void reserve_plans(Context& ctx, size_t n);
void compute_diagonal_elements(Context& ctx, const DTensor& L, const DTensor& R, DTensor& diag);

// src/renormalize.hpp:57-95 (merged operator); result allocated by the callee
std::unique_ptr<DTensor> renormalize(Context& ctx, bool forward, const DTensor& opr0, const DTensor& bra,
                                     const DTensor& ket);

// src/optimize.hpp:273-368 (one operator group); mpo must carry host data
std::unique_ptr<DTensor> compute_merged_operator(Context& ctx, bool forward, const DTensor& mpo,
                                                 const DTensor& opr);

// src/diagonalize.hpp:310-449 (single root)
double diagonalize(Context& ctx, const DTensor& L, const DTensor& R, const DTensor& diag, DTensor& wfnc,
                   double tol, DavidsonStats* stats);

// src/canonicalize.hpp:88-106 + include/btas/QSPARSE/QSTLAPACK.h:121-288
struct CanonResult {
  std::unique_ptr<DTensor> lmat, rmat;
  std::vector<std::pair<int, int>> kept;  // (sector, kept count) of the new bond
  double discarded = 0.0;
};
CanonResult canonicalize(Context& ctx, bool forward, const DTensor& wfnc, int M, double noise);
// src/canonicalize.hpp:11-24: the first n values of the sequence make_noise draws
// (a default-seeded std::mt19937 through std::uniform_real_distribution<double>(-1, 1)).
std::vector<double> noise_sequence(int64_t n);
// make_noise: a copy of wfnc plus noise times the noise array (null when noise < 1e-8,
// which leaves wfnc unchanged).  The noise array holds every allowed block whose
// sectors have a block in wfnc; each of its blocks holds the leading values of
// noise_sequence in row-major order, and blocks that wfnc lacks are added.
std::unique_ptr<DTensor> make_noise(Context& ctx, const DTensor& wfnc, double noise);
// Several independent canonicalisations sharing one solve (one Jacobi launch and one
// set of solver lanes for all their blocks, one read-back of the singular values).
struct CanonJob {
  bool forward;
  const DTensor* wfnc;
  int M;
};
std::vector<CanonResult> canonicalize_many(Context& ctx, const std::vector<CanonJob>& jobs);

// global top-M selection with a relative tie window (QSTLAPACK.h:204-232)
std::vector<int> select_kept(const std::vector<std::vector<double>>& svals, int M, double tie_rtol,
                             double* discarded);

// merged wavefunction psi[A,B] from lwfn[l,n,m] * rwfn[m,n',r] (src/optimize.hpp:542-557)
struct WaveMerge {
  MergeInfo ql, qr;
};
WaveMerge wave_merge_infos(const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr, const DTensor& ropr);
std::unique_ptr<DTensor> merge_wave(Context& ctx, const WaveMerge& wm, const DTensor& lwfn, const DTensor& rwfn);
// merge_wave in two halves: the plan by layouts (safe on planning threads), the run
std::unique_ptr<WavePlan> plan_merge_wave(Context& ctx, const WaveMerge& wm, const Tensor& lwfn, const Tensor& rwfn);
std::unique_ptr<DTensor> run_merge_wave(Context& ctx, WavePlan& wp, const DTensor& lwfn, const DTensor& rwfn);
std::unique_ptr<DTensor> expand_rows(Context& ctx, const MergeInfo& info, const DTensor& b);
std::unique_ptr<DTensor> expand_cols(Context& ctx, const DTensor& b, const MergeInfo& info);
// QSTmerge column merge of the trailing indices (include/btas/QSPARSE/QSTmerge.h:85-140)
std::unique_ptr<DTensor> merge_cols(Context& ctx, const DTensor& a, const MergeInfo& info);
std::unique_ptr<DTensor> merge_rows(Context& ctx, const MergeInfo& info, const DTensor& a);

// btas::Gemm into an empty result (QSTBLAS.h:182-226)
std::unique_ptr<DTensor> gemm_new(Context& ctx, Trans ta, Trans tb, double alpha, const DTensor& a, const DTensor& b,
                                  int c_rank);
// btas::Normalize; returns the norm before scaling
double normalize_tensor(Context& ctx, DTensor& x);

// A copy of x in the block layout `tags` (ascending, a superset of x's blocks; the
// added blocks are zero).
std::unique_ptr<DTensor> relayout(Context& ctx, const DTensor& x, const std::vector<int64_t>& tags);
// y += alpha x (btas::Axpy, include/btas/SPARSE/STBLAS.h:133-145): same sectors; the
// blocks of x that y lacks are added to y (y is replaced by a grown copy then).
void accumulate_into(Context& ctx, double alpha, const DTensor& x, std::unique_ptr<DTensor>& y);
// The other compute_sigma_vector overloads (src/compute_sigma_vector.hpp), results
// allocated by the callee: one-site with the site MPO (:9-22), two-site four-index
// (:53-70), and lopr wfn ropr^T with two-index overlap operators for wfn of 2, 3 or 4
// indices (:24-35, :72-83, :98-109).
std::unique_ptr<DTensor> sigma_onesite(Context& ctx, const DTensor& mpo, const DTensor& lopr, const DTensor& ropr,
                                       const DTensor& wfn);
std::unique_ptr<DTensor> sigma_twosite(Context& ctx, const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr,
                                       const DTensor& ropr, const DTensor& wfn);
std::unique_ptr<DTensor> sigma_overlap(Context& ctx, const DTensor& lopr, const DTensor& ropr, const DTensor& wfn);
// renormalize with the site MPO (src/renormalize.hpp:10-32) and of an overlap matrix
// (:35-54), results allocated by the callee
std::unique_ptr<DTensor> renormalize_mpo(Context& ctx, bool forward, const DTensor& mpo, const DTensor& opr0,
                                         const DTensor& bra, const DTensor& ket);
std::unique_ptr<DTensor> renormalize_overlap(Context& ctx, bool forward, const DTensor& sov0, const DTensor& bra,
                                             const DTensor& ket);
// compute_guesswave (src/compute_guesswave.hpp:11-38): forward C(i+1) = L(i)^+ C(i) R(i+1),
// backward C(i) = L(i) C(i+1) R(i+1)^+, result allocated by the callee
std::unique_ptr<DTensor> guesswave(Context& ctx, bool forward, const DTensor& mps0, const DTensor& wfn0,
                                   const DTensor& mps1);
// compute_diagonal_elements, one-site (src/compute_diagonal_elements.hpp:10-32) and
// four-index two-site (:35-62): the diagonal on every allowed block of like's sectors
std::unique_ptr<DTensor> diagonal_onesite(Context& ctx, const DTensor& mpo, const DTensor& lopr, const DTensor& ropr,
                                          const DTensor& like);
std::unique_ptr<DTensor> diagonal_twosite(Context& ctx, const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr,
                                          const DTensor& ropr, const DTensor& like);

// One bond (src/optimize.hpp:495-651)
struct BondStats {
  double energy = 0.0;
  DavidsonStats dav;
  double t_merge = 0, t_diag = 0, t_davidson = 0, t_svd = 0, t_renorm = 0;
  double sigma_flops = 0.0;
};
struct BondOut {
  std::unique_ptr<DTensor> env, lwfn, rwfn;
  BondStats stats;
};
BondOut optimize_twosite_merged(Context& ctx, bool forward, const DTensor& lmpo, const DTensor& rmpo,
                                const DTensor& lopr, const DTensor& ropr, const DTensor& lwfn,
                                const DTensor& rwfn, double tole, int M,
                                double noise = 0.0);

// --- batched steps over independent problems (batch.cpp) --------------------
// Lowest eigenpairs of independent effective Hamiltonians, Davidson in lockstep with
// one grouped tensor-core H_eff*psi launch (split precision) for all of them.
std::vector<double> diagonalize_batch(Context& ctx, const std::vector<const DTensor*>& L,
                                      const std::vector<const DTensor*>& R, const std::vector<const DTensor*>& diag,
                                      const std::vector<DTensor*>& psi, double tol, std::vector<DavidsonStats>& stats);
struct BondArgs {
  bool forward = true;
  const DTensor *lmpo = nullptr, *rmpo = nullptr, *lopr = nullptr, *ropr = nullptr, *lwfn = nullptr,
                *rwfn = nullptr;
  int M = 0;
  double noise = 0.0;  // make_noise before the truncation (src/canonicalize.hpp:95)
};
// optimize_twosite_merged for every bond of `args` (independent problems), their
// Davidson iterations batched.
std::vector<BondOut> optimize_twosite_merged_batch(Context& ctx, const std::vector<BondArgs>& args, double tole);

}  // namespace mpsxx
