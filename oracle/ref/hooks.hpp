// Force-included (g++ -include) into the reference's DMRG translation units and into
// the oracle's reference harness.  Oracle test infrastructure only.
//
// 1. Block-task recording.  ST_Gemm_thread (include/btas/SPARSE/STBLAS.h:297-359)
//    hands its task list to parallel_call (include/btas/SPARSE/T_arguments.h:585-600)
//    through an unqualified call.  The overload below is more specialised than the
//    reference's template, so that call resolves here for every Gemm.  When a sink is
//    set it copies the list in enumeration order (result block, ordered operand-block
//    pairs, as raw block addresses the harness maps back to tags); it then runs the
//    tasks as the reference does: sorted by the FLOPS_ proxy, largest first, over an
//    OpenMP guided loop.
// 2. The Davidson functors' operator() (src/diagonalize.hpp:65-80, 155-170, 239-254)
//    is declared `double` but never returns, which is undefined behaviour that GCC
//    turns into falling through at -O2.  The explicit specialisations below for the
//    fermion quantum number do what those bodies do (sigma over every operator group,
//    then the projections of the lower roots) and return 0; callers ignore the value.
#ifndef MPSXX_REF_HOOKS_HPP
#define MPSXX_REF_HOOKS_HPP

#include <algorithm>
#include <functional>
#include <tuple>
#include <utility>
#include <vector>

#include <btas/SPARSE/T_arguments.h>

namespace mpsxx_ref {
struct TaskRecord {
  const void* c;
  std::vector<std::pair<const void*, const void*>> pairs;
  double flops;  // sum of 2*m*n*k over the pairs, from the operand shapes
};
// Non-null: every Gemm's task list is appended here before it runs.
extern std::vector<std::vector<TaskRecord>>* task_sink;
}  // namespace mpsxx_ref

namespace btas {

template <typename T, size_t L, size_t M, size_t N>
void parallel_call(std::vector<Gemm_arguments<T, L, M, N>>& task) {
  using std::get;
  if (mpsxx_ref::task_sink) {
    std::vector<mpsxx_ref::TaskRecord> list;
    list.reserve(task.size());
    for (const auto& t : task) {
      mpsxx_ref::TaskRecord r;
      r.c = get<2>(t).get();
      r.flops = 0.0;
      const size_t np = get<0>(t).size();
      const double cn = static_cast<double>(get<2>(t)->size());
      for (size_t i = 0; i < np; ++i) {
        r.pairs.emplace_back(get<0>(t)[i].get(), get<1>(t)[i].get());
        // the contracted extent k = size(A) * size(B) / size(C) for a plain matrix product
        const double a = static_cast<double>(get<0>(t)[i]->size());
        const double b = static_cast<double>(get<1>(t)[i]->size());
        r.flops += cn > 0 ? 2.0 * std::sqrt(a * b * cn) : 0.0;
      }
      list.push_back(std::move(r));
    }
    mpsxx_ref::task_sink->push_back(std::move(list));
  }
  std::sort(task.begin(), task.end(), std::greater<Gemm_arguments<T, L, M, N>>());
  const size_t n = task.size();
#pragma omp parallel for schedule(guided)
  for (size_t i = 0; i < n; ++i) task[i].call();
}

}  // namespace btas

#include "fermion.h"
#include "diagonalize.hpp"
#include "optimize.hpp"

namespace mpsxx {
namespace Davidson {

template <>
inline double Functor<2, fermion>::operator()(const MPS_type& c, MPS_type& v) const {
  Communicator world;
  for (size_t g = 0; g < pLOp_->size(); ++g) compute_sigma_vector((*pLOp_)[g], (*pROp_)[g], c, v);
  for (size_t k = 0; k + 1 < N_; ++k) {
    const double hk = btas::Dotc(H_[k], c), sk = btas::Dotc(S_[k], c);
    btas::Axpy(-hk, S_[k], v);
    btas::Axpy(-sk, H_[k], v);
    if (world.rank() == 0) btas::Axpy(E_[k] * sk, S_[k], v);
  }
  return 0.0;
}

template <>
inline double Functor<3, fermion>::operator()(const MPS_type& c, MPS_type& v) const {
  Communicator world;
  for (size_t g = 0; g < pMPO_->size(); ++g) compute_sigma_vector((*pMPO_)[g], (*pLOp_)[g], (*pROp_)[g], c, v);
  for (size_t k = 0; k + 1 < N_; ++k) {
    const double hk = btas::Dotc(H_[k], c), sk = btas::Dotc(S_[k], c);
    btas::Axpy(-hk, S_[k], v);
    btas::Axpy(-sk, H_[k], v);
    if (world.rank() == 0) btas::Axpy(E_[k] * sk, S_[k], v);
  }
  return 0.0;
}

template <>
inline double Functor<4, fermion>::operator()(const MPS_type& c, MPS_type& v) const {
  Communicator world;
  for (size_t g = 0; g < pLMPO_->size(); ++g)
    compute_sigma_vector((*pLMPO_)[g], (*pRMPO_)[g], (*pLOp_)[g], (*pROp_)[g], c, v);
  for (size_t k = 0; k + 1 < N_; ++k) {
    const double hk = btas::Dotc(H_[k], c), sk = btas::Dotc(S_[k], c);
    btas::Axpy(-hk, S_[k], v);
    btas::Axpy(-sk, H_[k], v);
    if (world.rank() == 0) btas::Axpy(E_[k] * sk, S_[k], v);
  }
  return 0.0;
}

}  // namespace Davidson

// 3. Bond dumps.  A non-template overload for the fermion quantum number is preferred
//    over the template optimize_twosite_merged (src/optimize.hpp:495-651) at the call
//    in make_sweep (src/make_sweep.cpp:112,215).  It calls the template unchanged;
//    with MPSXX_REF_DUMP=<dir> it first writes the bond's inputs and afterwards its
//    outputs to <dir>/bond_NNNNN/ (qsd_io.hpp files, meta.txt).
double optimize_twosite_merged(bool forward, const std::vector<double>& E,
                               const std::vector<btas::QSTArray<double, 4, fermion>>& lmpo,
                               const std::vector<btas::QSTArray<double, 4, fermion>>& rmpo,
                               std::vector<std::vector<btas::QSTArray<double, 3, fermion>>>& lHopr,
                               std::vector<std::vector<btas::QSTArray<double, 3, fermion>>>& rHopr,
                               std::vector<btas::QSTArray<double, 2, fermion>>& lSopr,
                               std::vector<btas::QSTArray<double, 2, fermion>>& rSopr,
                               std::vector<btas::QSTArray<double, 3, fermion>>& kMps,
                               std::vector<btas::QSTArray<double, 3, fermion>>& lWfnc,
                               std::vector<btas::QSTArray<double, 3, fermion>>& rWfnc, const double& tole,
                               const int& M, const double& noise = 0.0);

}  // namespace mpsxx

#endif
