// C++ drop-in surface of the GB300 two-site DMRG hot path.
//
// The functions keep the reference's names, argument order and meaning
// (src/compute_sigma_vector.hpp:85-96, src/renormalize.hpp:57-95,
// src/compute_diagonal_elements.hpp:65-80, src/diagonalize.hpp:310-449,
// src/canonicalize.hpp:88-106) over gb300::QSDArray, a device-resident
// block-sparse tensor with the data model of btas::QSTArray<double,N,fermion>.
// Failures throw std::runtime_error with the reference's messages, as BTAS_THROW
// does (include/btas/common/btas.h:19-20).  Every call forwards to the C ABI in
// mpsxx_gb300.h; link with -lmpsxx_gb300.
#ifndef MPSXX_GB300_HPP
#define MPSXX_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mpsxx_gb300.h"

namespace mpsxx {
namespace gb300 {

inline void check(int rc) {
  if (rc != MPSXX_OK) throw std::runtime_error(std::string(mpsxx_last_error()));
}

// One device and one stream (nullptr: the context creates its own stream).
class Context {
 public:
  explicit Context(int device = 0, void* stream = nullptr) { check(mpsxx_context_create(device, stream, &h_)); }
  ~Context() {
    if (h_) mpsxx_context_destroy(h_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  mpsxx_context* get() const { return h_; }
  void set_precision(int p) { check(mpsxx_context_set_precision(h_, p)); }
  void set_truncation(double tie_rtol) { check(mpsxx_context_set_truncation(h_, tie_rtol)); }

 private:
  mpsxx_context* h_ = nullptr;
};

// Quantum number (particle number, 2*Sz) and dimension of one sector of an index.
struct Sector {
  int p, s, dim;
};

// Block-sparse tensor: q_total, per-index sectors, stored block tags (row-major
// sparse index, ascending), device data packed in tag order.  ctx == nullptr makes a
// host-only descriptor (block structure only), enough for the planner.
class QSDArray {
 public:
  QSDArray() = default;
  QSDArray(Context* ctx, int p_total, int s_total, const std::vector<std::vector<Sector>>& shape,
           const std::vector<int64_t>* tags = nullptr) {
    std::vector<int> nsec, qn, dims;
    for (const auto& idx : shape) {
      nsec.push_back(static_cast<int>(idx.size()));
      for (const auto& s : idx) {
        qn.push_back(s.p);
        qn.push_back(s.s);
        dims.push_back(s.dim);
      }
    }
    const int q[2] = {p_total, s_total};
    check(mpsxx_tensor_create(ctx ? ctx->get() : nullptr, static_cast<int>(shape.size()), q, nsec.data(),
                              qn.empty() ? nullptr : qn.data(), dims.empty() ? nullptr : dims.data(),
                              tags ? static_cast<int64_t>(tags->size()) : -1, tags ? tags->data() : nullptr, &h_));
  }
  static QSDArray adopt(mpsxx_tensor* h) {
    QSDArray a;
    a.h_ = h;
    return a;
  }
  ~QSDArray() { reset(); }
  QSDArray(const QSDArray&) = delete;
  QSDArray& operator=(const QSDArray&) = delete;
  QSDArray(QSDArray&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  QSDArray& operator=(QSDArray&& o) noexcept {
    if (this != &o) {
      reset();
      h_ = o.h_;
      o.h_ = nullptr;
    }
    return *this;
  }
  void reset() {
    if (h_) mpsxx_tensor_destroy(h_);
    h_ = nullptr;
  }
  bool empty() const { return h_ == nullptr; }
  mpsxx_tensor* get() const { return h_; }
  int64_t nnz() const {
    int64_t n = 0;
    check(mpsxx_tensor_info(h_, nullptr, nullptr, nullptr, &n));
    return n;
  }
  int64_t nblocks() const {
    int64_t n = 0;
    check(mpsxx_tensor_info(h_, nullptr, nullptr, &n, nullptr));
    return n;
  }
  int rank() const {
    int r = 0;
    check(mpsxx_tensor_info(h_, &r, nullptr, nullptr, nullptr));
    return r;
  }
  void upload(const double* host) { check(mpsxx_tensor_upload(h_, host)); }
  void download(double* host) const { check(mpsxx_tensor_download(h_, host)); }

 private:
  mpsxx_tensor* h_ = nullptr;
};

// --- the reference's call surface ------------------------------------------

namespace detail {
// the allocate-or-accumulate output of the rank overloads: an empty sgv0 receives the
// result, a non-empty one is added to (and grows by any missing blocks)
template <class F>
inline void into(QSDArray& sgv0, F call) {
  mpsxx_tensor* h = sgv0.get();
  check(call(&h));
  if (sgv0.empty()) sgv0 = QSDArray::adopt(h);
}
}  // namespace detail

// sgv0 += H_eff * wfn0 for merged operators; an empty sgv0 is created with wfn0's
// layout first.  With two-index (overlap) operators: sgv0 += lopr wfn0 ropr^T
// (src/compute_sigma_vector.hpp:24-35, 72-83, 98-109), for wfn0 of 2, 3 or 4 indices.
inline void compute_sigma_vector(Context& ctx, const QSDArray& lopr, const QSDArray& ropr, const QSDArray& wfn0,
                                 QSDArray& sgv0) {
  if (lopr.rank() == 2) {
    detail::into(sgv0, [&](mpsxx_tensor** o) {
      return mpsxx_compute_sigma_vector_overlap(ctx.get(), lopr.get(), ropr.get(), wfn0.get(), o);
    });
    return;
  }
  if (sgv0.empty()) {
    mpsxx_tensor* h = nullptr;
    check(mpsxx_tensor_create_like(ctx.get(), wfn0.get(), &h));
    sgv0 = QSDArray::adopt(h);
  }
  check(mpsxx_compute_sigma_vector(ctx.get(), lopr.get(), ropr.get(), wfn0.get(), sgv0.get()));
}

// One-site: sgv0 (+)= H wfn0 with the site MPO (src/compute_sigma_vector.hpp:9-22).
inline void compute_sigma_vector(Context& ctx, const QSDArray& mpo0, const QSDArray& lopr, const QSDArray& ropr,
                                 const QSDArray& wfn0, QSDArray& sgv0) {
  detail::into(sgv0, [&](mpsxx_tensor** o) {
    return mpsxx_compute_sigma_vector_onesite(ctx.get(), mpo0.get(), lopr.get(), ropr.get(), wfn0.get(), o);
  });
}

// Two-site, four-index wavefunction (src/compute_sigma_vector.hpp:53-70).
inline void compute_sigma_vector(Context& ctx, const QSDArray& lmpo, const QSDArray& rmpo, const QSDArray& lopr,
                                 const QSDArray& ropr, const QSDArray& wfn0, QSDArray& sgv0) {
  detail::into(sgv0, [&](mpsxx_tensor** o) {
    return mpsxx_compute_sigma_vector_twosite(ctx.get(), lmpo.get(), rmpo.get(), lopr.get(), ropr.get(),
                                              wfn0.get(), o);
  });
}

// diag += sum_w lopr[A,w,A] ropr[B,w,B] on diag's blocks.
inline void compute_diagonal_elements(Context& ctx, const QSDArray& lopr, const QSDArray& ropr, QSDArray& diag) {
  check(mpsxx_compute_diagonal_elements(ctx.get(), lopr.get(), ropr.get(), diag.get()));
}

// One-site and four-index two-site diagonals (src/compute_diagonal_elements.hpp:10-62):
// diag = the diagonal on every allowed block of diag's sectors; as the reference's
// Copy(scr, diag, 1), what diag held before is dropped.
inline void compute_diagonal_elements(Context& ctx, const QSDArray& mpo0, const QSDArray& lopr, const QSDArray& ropr,
                                      QSDArray& diag) {
  check(mpsxx_compute_diagonal_elements_onesite(ctx.get(), mpo0.get(), lopr.get(), ropr.get(), diag.get()));
}
inline void compute_diagonal_elements(Context& ctx, const QSDArray& lmpo, const QSDArray& rmpo, const QSDArray& lopr,
                                      const QSDArray& ropr, QSDArray& diag) {
  check(mpsxx_compute_diagonal_elements_twosite(ctx.get(), lmpo.get(), rmpo.get(), lopr.get(), ropr.get(),
                                                diag.get()));
}

// wfn1 += guess wavefunction of the next site (src/compute_guesswave.hpp:11-38): forward
// (L(i), C(i), R(i+1)) -> C(i+1), backward (R(i+1), C(i+1), L(i)) -> C(i); an empty wfn1
// receives the result.
inline void compute_guesswave(Context& ctx, bool forward, const QSDArray& mps0, const QSDArray& wfn0,
                              const QSDArray& mps1, QSDArray& wfn1) {
  detail::into(wfn1, [&](mpsxx_tensor** o) {
    return mpsxx_compute_guesswave(ctx.get(), forward ? 1 : 0, mps0.get(), wfn0.get(), mps1.get(), o);
  });
}

// opr1 = renormalised merged operator (allocated here, as a Gemm into an empty array).
// With a two-index opr0 it renormalises an overlap matrix (src/renormalize.hpp:35-54),
// allocate-or-accumulate.
inline void renormalize(Context& ctx, bool forward, const QSDArray& opr0, const QSDArray& bra0, const QSDArray& ket0,
                        QSDArray& opr1) {
  if (opr0.rank() == 2) {
    detail::into(opr1, [&](mpsxx_tensor** o) {
      return mpsxx_renormalize_overlap(ctx.get(), forward ? 1 : 0, opr0.get(), bra0.get(), ket0.get(), o);
    });
    return;
  }
  mpsxx_tensor* h = nullptr;
  check(mpsxx_renormalize(ctx.get(), forward ? 1 : 0, opr0.get(), bra0.get(), ket0.get(), &h));
  opr1 = QSDArray::adopt(h);
}

// renormalize with the site MPO (src/renormalize.hpp:10-32), allocate-or-accumulate.
inline void renormalize(Context& ctx, bool forward, const QSDArray& mpo0, const QSDArray& opr0, const QSDArray& bra0,
                        const QSDArray& ket0, QSDArray& opr1) {
  detail::into(opr1, [&](mpsxx_tensor** o) {
    return mpsxx_renormalize_mpo(ctx.get(), forward ? 1 : 0, mpo0.get(), opr0.get(), bra0.get(), ket0.get(), o);
  });
}

namespace Davidson {
// Lowest eigenpair; wfnc is overwritten by the Ritz vector, the Ritz value returned.
inline double diagonalize(Context& ctx, const QSDArray& lopr, const QSDArray& ropr, const QSDArray& diag,
                          QSDArray& wfnc, double tolerance = 1.0e-8) {
  double e = 0.0;
  check(mpsxx_diagonalize(ctx.get(), lopr.get(), ropr.get(), diag.get(), wfnc.get(), tolerance, &e, nullptr));
  return e;
}
}  // namespace Davidson

// wfnc += noise * noise array, in place; nothing when noise < 1e-8 (src/canonicalize.hpp:11-24).
inline void make_noise(Context& ctx, QSDArray& wfnc, double noise) {
  check(mpsxx_make_noise(ctx.get(), wfnc.get(), noise));
}

// Truncated SVD: forward -> lmat = U, rmat = s V^T; backward -> lmat = U s, rmat = V^T.
inline void canonicalize(Context& ctx, bool forward, const QSDArray& wfnc, QSDArray& lmat, QSDArray& rmat,
                         int M = 0, double noise = 0.0) {
  mpsxx_tensor *l = nullptr, *r = nullptr;
  check(mpsxx_canonicalize(ctx.get(), forward ? 1 : 0, wfnc.get(), M, noise, &l, &r));
  lmat = QSDArray::adopt(l);
  rmat = QSDArray::adopt(r);
}

// Reference block-task list of btas::Gemm (host only): (c tag, [(a tag, b tag)]).
inline std::vector<std::pair<int64_t, std::vector<std::pair<int64_t, int64_t>>>> gemm_tasks(int transa, int transb,
                                                                                               const QSDArray& a,
                                                                                               const QSDArray& b,
                                                                                               int c_rank) {
  int64_t nt = 0, np = 0;
  check(mpsxx_gemm_tasks(transa, transb, a.get(), b.get(), c_rank, &nt, &np, nullptr, nullptr, nullptr, nullptr));
  std::vector<int64_t> ct(nt), pp(nt + 1), at(np), bt(np);
  check(mpsxx_gemm_tasks(transa, transb, a.get(), b.get(), c_rank, &nt, &np, ct.data(), pp.data(), at.data(),
                         bt.data()));
  std::vector<std::pair<int64_t, std::vector<std::pair<int64_t, int64_t>>>> out(nt);
  for (int64_t i = 0; i < nt; ++i) {
    out[i].first = ct[i];
    for (int64_t p = pp[i]; p < pp[i + 1]; ++p) out[i].second.emplace_back(at[p], bt[p]);
  }
  return out;
}

}  // namespace gb300
}  // namespace mpsxx

#endif  // MPSXX_GB300_HPP
