// The other rank overloads of the reference's hot-path functions on the device path,
// and the block-layout helpers they share with make_noise:
//   compute_sigma_vector (src/compute_sigma_vector.hpp)
//     one-site   sgv[l,n,r]    += H wfn with the site MPO            (:9-22)
//     two-site   sgv[l,n,n',r] += H wfn with both site MPOs          (:53-70)
//     overlap    sgv           += lS wfn rS^T for two-index S blocks  (:24-35, :72-83, :98-109)
//   renormalize (src/renormalize.hpp): with the site MPO (:10-32), overlap (:35-54)
//   compute_diagonal_elements (src/compute_diagonal_elements.hpp): one-site (:10-32),
//     two-site four-index (:35-62)
//   compute_guesswave (src/compute_guesswave.hpp:11-38): the centre moved one site
// The H forms run as the merged products: the block operator is merged with its site
// MPO (compute_merged_operator), the site tensors are merged over the same index
// pairs, the merged kernels run (on every allowed merged block where the result's
// layout is not given), and results are expanded back.  The merged sectors follow
// first appearance in packed order, so merging a tensor's ket sectors and the
// operator's (negated) ket sectors gives the same sector order.  The overlap forms
// are the reference's two Gemms.
#include <algorithm>
#include <iterator>

#include "engine.hpp"

namespace mpsxx {

std::unique_ptr<DTensor> relayout(Context& ctx, const DTensor& x, const std::vector<int64_t>& tags) {
  cudaStream_t st = ctx.stream;
  auto out = std::make_unique<DTensor>();
  static_cast<Tensor&>(*out) = static_cast<const Tensor&>(x);
  out->d = nullptr;
  out->own = false;
  out->ctx = &ctx;
  const bool same = tags == x.tags;
  if (!same) out->set_blocks(tags);
  out->alloc_device(st, !same);
  if (same) {
    if (x.nnz)
      cuda_check(cudaMemcpyAsync(out->d, x.d, x.nnz * sizeof(double), cudaMemcpyDeviceToDevice, st), "relayout copy");
    return out;
  }
  std::vector<DCopy> cp;
  for (size_t b = 0; b < x.tags.size(); ++b) {
    const int32_t s = out->find(x.tags[b]);
    if (s < 0) throw Error(kInternal, "relayout: a block of the source is not in the new layout");
    const int64_t n = x.block_size(static_cast<int32_t>(b));
    if (n > 0x7fffffff) throw Error(kInvalidArgument, "relayout: block too large");
    if (n > 0)
      cp.push_back(DCopy{out->offsets[s], x.offsets[b], 1, static_cast<int>(n), static_cast<int>(n),
                         static_cast<int>(n), 1.0});
  }
  if (!cp.empty()) {
    DevArray<DCopy> dcp;
    dcp.upload(cp, st);
    launch_copy(dcp.get(), static_cast<int>(cp.size()), x.d, out->d, 0, st);
    ctx.kernel_launches += 1;
  }
  return out;
}

void accumulate_into(Context& ctx, double alpha, const DTensor& x, std::unique_ptr<DTensor>& y) {
  if (x.sh.rank != y->sh.rank || !(x.sh.q == y->sh.q))
    throw Error(kQShapeMismatch, "Axpy(QSPARSE): x and y must have the same quantum number.");
  for (int i = 0; i < x.sh.rank; ++i)
    if (x.sh.qshape[i] != y->sh.qshape[i] || x.sh.dshape[i] != y->sh.dshape[i])
      throw Error(kQShapeMismatch, "Axpy(QSPARSE): x and y must have the same quantum shape.");
  std::vector<int64_t> u;
  std::set_union(y->tags.begin(), y->tags.end(), x.tags.begin(), x.tags.end(), std::back_inserter(u));
  if (u.size() != y->tags.size()) y = relayout(ctx, *y, u);
  std::vector<DCopy> cp;
  for (size_t b = 0; b < x.tags.size(); ++b) {
    const int32_t s = y->find(x.tags[b]);
    const int64_t n = x.block_size(static_cast<int32_t>(b));
    if (n > 0x7fffffff) throw Error(kInvalidArgument, "accumulate: block too large");
    if (n > 0) cp.push_back(DCopy{y->offsets[s], x.offsets[b], 1, static_cast<int>(n), 0, 0, alpha});
  }
  if (cp.empty()) return;
  DevArray<DCopy> dcp;
  dcp.upload(cp, ctx.stream);
  launch_copy(dcp.get(), static_cast<int>(cp.size()), x.d, y->d, 1, ctx.stream);
  ctx.kernel_launches += 1;
}

namespace {
// psi with every allowed block of its merged shape (zero where wfn had no data), so
// that the merged product reaches every block H * wfn can have
std::unique_ptr<DTensor> all_allowed(Context& ctx, const DTensor& psi) {
  Tensor full;
  full.sh = psi.sh;
  full.allocate_allowed();
  return relayout(ctx, psi, full.tags);
}

std::unique_ptr<DTensor> zeros_like(Context& ctx, const DTensor& x) {
  auto z = std::make_unique<DTensor>();
  static_cast<Tensor&>(*z) = static_cast<const Tensor&>(x);
  z->d = nullptr;
  z->own = false;
  z->ctx = &ctx;
  z->alloc_device(ctx.stream, true);
  return z;
}

void need_rank(const DTensor& t, int r, const char* what) {
  if (t.sh.rank != r) throw Error(kInvalidArgument, what);
}
}  // namespace

std::unique_ptr<DTensor> sigma_onesite(Context& ctx, const DTensor& mpo, const DTensor& lopr, const DTensor& ropr,
                                       const DTensor& wfn) {
  need_rank(mpo, 4, "compute_sigma_vector: the site MPO must have 4 indices");
  need_rank(lopr, 3, "compute_sigma_vector: the block operators must have 3 indices");
  need_rank(ropr, 3, "compute_sigma_vector: the block operators must have 3 indices");
  need_rank(wfn, 3, "compute_sigma_vector: the one-site wavefunction must have 3 indices");
  auto mL = compute_merged_operator(ctx, true, mpo, lopr);
  const MergeInfo rows({wfn.sh.qshape[0], wfn.sh.qshape[1]}, {wfn.sh.dshape[0], wfn.sh.dshape[1]});
  auto psi = all_allowed(ctx, *merge_rows(ctx, rows, wfn));
  auto sig = zeros_like(ctx, *psi);
  compute_sigma_vector(ctx, *mL, ropr, *psi, *sig);
  return expand_rows(ctx, rows, *sig);
}

std::unique_ptr<DTensor> sigma_twosite(Context& ctx, const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr,
                                       const DTensor& ropr, const DTensor& wfn) {
  need_rank(lmpo, 4, "compute_sigma_vector: the site MPOs must have 4 indices");
  need_rank(rmpo, 4, "compute_sigma_vector: the site MPOs must have 4 indices");
  need_rank(lopr, 3, "compute_sigma_vector: the block operators must have 3 indices");
  need_rank(ropr, 3, "compute_sigma_vector: the block operators must have 3 indices");
  need_rank(wfn, 4, "compute_sigma_vector: the two-site wavefunction must have 4 indices");
  auto mL = compute_merged_operator(ctx, true, lmpo, lopr);
  auto mR = compute_merged_operator(ctx, false, rmpo, ropr);
  const MergeInfo rows({wfn.sh.qshape[0], wfn.sh.qshape[1]}, {wfn.sh.dshape[0], wfn.sh.dshape[1]});
  const MergeInfo cols({wfn.sh.qshape[2], wfn.sh.qshape[3]}, {wfn.sh.dshape[2], wfn.sh.dshape[3]});
  auto psi = all_allowed(ctx, *merge_rows(ctx, rows, *merge_cols(ctx, wfn, cols)));
  auto sig = zeros_like(ctx, *psi);
  compute_sigma_vector(ctx, *mL, *mR, *psi, *sig);
  return expand_cols(ctx, *expand_rows(ctx, rows, *sig), cols);
}

namespace {
// bra0.conjugate() (a view of the same data with every quantum number negated)
std::unique_ptr<DTensor> conjugate_view(const DTensor& x) {
  auto v = std::make_unique<DTensor>();
  static_cast<Tensor&>(*v) = static_cast<const Tensor&>(x);
  v->sh = x.sh.conjugate();
  v->own = false;
  v->ctx = x.ctx;
  v->set_blocks(x.tags);  // same blocks, layout identity of the conjugated shape
  v->data_version = next_data_version();
  return v;
}
}  // namespace

std::unique_ptr<DTensor> renormalize_mpo(Context& ctx, bool forward, const DTensor& mpo, const DTensor& opr0,
                                         const DTensor& bra, const DTensor& ket) {
  if (mpo.sh.rank != 4 || opr0.sh.rank != 3 || bra.sh.rank != 3 || ket.sh.rank != 3)
    throw Error(kInvalidArgument, "renormalize: site MPO of 4 indices, operator and site tensors of 3");
  auto mop = compute_merged_operator(ctx, forward, mpo, opr0);
  if (forward) {
    const MergeInfo rb({bra.sh.qshape[0], bra.sh.qshape[1]}, {bra.sh.dshape[0], bra.sh.dshape[1]});
    const MergeInfo rk({ket.sh.qshape[0], ket.sh.qshape[1]}, {ket.sh.dshape[0], ket.sh.dshape[1]});
    return renormalize(ctx, true, *mop, *merge_rows(ctx, rb, bra), *merge_rows(ctx, rk, ket));
  }
  const MergeInfo cb({bra.sh.qshape[1], bra.sh.qshape[2]}, {bra.sh.dshape[1], bra.sh.dshape[2]});
  const MergeInfo ck({ket.sh.qshape[1], ket.sh.qshape[2]}, {ket.sh.dshape[1], ket.sh.dshape[2]});
  return renormalize(ctx, false, *mop, *merge_cols(ctx, bra, cb), *merge_cols(ctx, ket, ck));
}

std::unique_ptr<DTensor> renormalize_overlap(Context& ctx, bool forward, const DTensor& sov0, const DTensor& bra,
                                             const DTensor& ket) {
  if (sov0.sh.rank != 2 || bra.sh.rank != 3 || ket.sh.rank != 3)
    throw Error(kInvalidArgument, "renormalize: overlap matrix of 2 indices, site tensors of 3");
  auto cbra = conjugate_view(bra);
  if (forward) {
    auto scr1 = gemm_new(ctx, kTrans, kNoTrans, 1.0, sov0, *cbra, 3);
    return gemm_new(ctx, kTrans, kNoTrans, 1.0, *scr1, ket, 2);
  }
  auto scr1 = gemm_new(ctx, kNoTrans, kNoTrans, 1.0, *cbra, sov0, 3);
  return gemm_new(ctx, kNoTrans, kTrans, 1.0, *scr1, ket, 2);
}

std::unique_ptr<DTensor> guesswave(Context& ctx, bool forward, const DTensor& mps0, const DTensor& wfn0,
                                   const DTensor& mps1) {
  if (mps0.sh.rank != 3 || wfn0.sh.rank != 3 || mps1.sh.rank != 3)
    throw Error(kInvalidArgument, "compute_guesswave: site tensors of 3 indices");
  // ConjTrans of a real QSDArray = Trans of its conjugate (negated quantum numbers,
  // same blocks and data): btas_contract_qshape.h takes -q for ConjTrans, the dense
  // layer treats it as Trans, and ST_Gemm_thread enumerates both alike
  auto c0 = conjugate_view(mps0);
  if (forward) {
    auto gmat = gemm_new(ctx, kTrans, kNoTrans, 1.0, *c0, wfn0, 2);
    return gemm_new(ctx, kNoTrans, kNoTrans, 1.0, *gmat, mps1, 3);
  }
  auto gmat = gemm_new(ctx, kNoTrans, kTrans, 1.0, wfn0, *c0, 2);
  return gemm_new(ctx, kNoTrans, kNoTrans, 1.0, mps1, *gmat, 3);
}

std::unique_ptr<DTensor> diagonal_onesite(Context& ctx, const DTensor& mpo, const DTensor& lopr, const DTensor& ropr,
                                          const DTensor& like) {
  need_rank(mpo, 4, "compute_diagonal_elements: the site MPO must have 4 indices");
  need_rank(like, 3, "compute_diagonal_elements: the one-site diagonal must have 3 indices");
  auto mL = compute_merged_operator(ctx, true, mpo, lopr);
  const MergeInfo rows({like.sh.qshape[0], like.sh.qshape[1]}, {like.sh.dshape[0], like.sh.dshape[1]});
  auto d = zeros_like(ctx, *all_allowed(ctx, *merge_rows(ctx, rows, like)));
  compute_diagonal_elements(ctx, *mL, ropr, *d);
  return expand_rows(ctx, rows, *d);
}

std::unique_ptr<DTensor> diagonal_twosite(Context& ctx, const DTensor& lmpo, const DTensor& rmpo, const DTensor& lopr,
                                          const DTensor& ropr, const DTensor& like) {
  need_rank(lmpo, 4, "compute_diagonal_elements: the site MPOs must have 4 indices");
  need_rank(rmpo, 4, "compute_diagonal_elements: the site MPOs must have 4 indices");
  need_rank(like, 4, "compute_diagonal_elements: the two-site diagonal must have 4 indices");
  auto mL = compute_merged_operator(ctx, true, lmpo, lopr);
  auto mR = compute_merged_operator(ctx, false, rmpo, ropr);
  const MergeInfo rows({like.sh.qshape[0], like.sh.qshape[1]}, {like.sh.dshape[0], like.sh.dshape[1]});
  const MergeInfo cols({like.sh.qshape[2], like.sh.qshape[3]}, {like.sh.dshape[2], like.sh.dshape[3]});
  auto d = zeros_like(ctx, *all_allowed(ctx, *merge_rows(ctx, rows, *merge_cols(ctx, like, cols))));
  compute_diagonal_elements(ctx, *mL, *mR, *d);
  return expand_cols(ctx, *expand_rows(ctx, rows, *d), cols);
}

std::unique_ptr<DTensor> sigma_overlap(Context& ctx, const DTensor& lopr, const DTensor& ropr, const DTensor& wfn) {
  need_rank(lopr, 2, "compute_sigma_vector: overlap block operators must have 2 indices");
  need_rank(ropr, 2, "compute_sigma_vector: overlap block operators must have 2 indices");
  if (wfn.sh.rank < 2 || wfn.sh.rank > 4) throw Error(kInvalidArgument, "compute_sigma_vector: wfn of 2 to 4 indices");
  auto scr1 = gemm_new(ctx, kNoTrans, kNoTrans, 1.0, lopr, wfn, wfn.sh.rank);
  return gemm_new(ctx, kNoTrans, kTrans, 1.0, *scr1, ropr, wfn.sh.rank);
}

}  // namespace mpsxx
