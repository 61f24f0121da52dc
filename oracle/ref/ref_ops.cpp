// Reference harness: runs the mpsxx reference's own hot-path functions on tensors
// read from qsd files and writes their results, so that the oracle and the CUDA path
// can be checked against the reference itself.  Oracle test infrastructure.
//
//   ref_ops.x ops <bond_dir>          bond inputs dumped by dmrg.x (hooks_impl.cpp) ->
//       mL, mR (compute_merged_operator, src/optimize.hpp:273-368), psi (the wavefunction
//       merge of src/optimize.hpp:542-557), sigma + both Gemm task lists
//       (src/compute_sigma_vector.hpp:85-96), diag (src/compute_diagonal_elements.hpp:152-179),
//       lmat/rmat (canonicalize, src/canonicalize.hpp:88-106, no noise) and the
//       renormalised operator + task lists (src/renormalize.hpp:57-95)
//   ref_ops.x time_sigma <dir> <steps> H_eff*psi on dir/{mL,mR,psi}.qsd: JSON timing line
//   ref_ops.x dump_mpo <prefix> <nsites> <outdir>  the site MPOs mpogen.x wrote
//       (src/make_qc_mpos.cpp:126-139, one operator group) as outdir/mpo_<i>.qsd
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>

#include <omp.h>

#include "hooks.hpp"
#include "qsd_io.hpp"
#include "canonicalize.hpp"
#include "compute_diagonal_elements.hpp"
#include "compute_sigma_vector.hpp"
#include "renormalize.hpp"
#include "fileio.h"

using QA2 = btas::QSTArray<double, 2, fermion>;
using QA3 = btas::QSTArray<double, 3, fermion>;
using QA4 = btas::QSTArray<double, 4, fermion>;
using mpsxx_ref::read_qsd;
using mpsxx_ref::TaskRecord;
using mpsxx_ref::write_qsd;

namespace {

// Block address -> tag of the tensor that owns it.
struct Registry {
  std::map<const void*, long> tag;
  template <size_t N>
  void add(const btas::QSTArray<double, N, fermion>& a) {
    for (auto it = a.begin(); it != a.end(); ++it)
      if (it->second) tag[it->second.get()] = it->first;
  }
  long operator()(const void* p) const {
    auto it = tag.find(p);
    return it == tag.end() ? -1 : it->second;
  }
};

// One line per task, in enumeration order: c_tag npairs a_tag b_tag ...
void write_tasks(std::ostream& os, const std::string& name, const std::vector<TaskRecord>& list, const Registry& ra,
                 const Registry& rb, const Registry& rc) {
  os << "gemm " << name << " " << list.size() << "\n";
  for (const auto& t : list) {
    os << rc(t.c) << " " << t.pairs.size();
    for (const auto& p : t.pairs) os << " " << ra(p.first) << " " << rb(p.second);
    os << "\n";
  }
}

std::map<std::string, std::string> read_meta(const std::string& path) {
  std::map<std::string, std::string> m;
  std::ifstream f(path);
  std::string k, v;
  while (f >> k >> v) m[k] = v;
  return m;
}

template <size_t N>
double max_abs_diff(const btas::QSTArray<double, N, fermion>& a, const btas::QSTArray<double, N, fermion>& b) {
  double d = 0.0;
  for (auto it = a.begin(); it != a.end(); ++it) {
    auto jt = b.find(it->first);
    for (size_t i = 0; i < it->second->size(); ++i) {
      const double y = jt == b.end() ? 0.0 : jt->second->data()[i];
      d = std::max(d, std::fabs(it->second->data()[i] - y));
    }
  }
  return d;
}

int run_ops(const std::string& dir) {
  auto meta = read_meta(dir + "/meta.txt");
  const bool forward = std::stoi(meta.at("forward")) != 0;
  const int M = std::stoi(meta.at("M"));
  QA4 lmpo, rmpo;
  QA3 lopr, ropr, lwfn, rwfn;
  QA2 lsopr, rsopr;
  read_qsd(dir + "/lmpo.qsd", lmpo);
  read_qsd(dir + "/rmpo.qsd", rmpo);
  read_qsd(dir + "/lopr.qsd", lopr);
  read_qsd(dir + "/ropr.qsd", ropr);
  read_qsd(dir + "/lsopr.qsd", lsopr);
  read_qsd(dir + "/rsopr.qsd", rsopr);
  read_qsd(dir + "/lwfn.qsd", lwfn);
  read_qsd(dir + "/rwfn.qsd", rwfn);

  // merged super-block operators
  std::vector<std::vector<QA3>> mLv, mRv, lH{{lopr}}, rH{{ropr}};
  std::vector<QA2> mSLv, mSRv, lS{lsopr}, rS{rsopr};
  mpsxx::compute_merged_operator(1, std::vector<QA4>{lmpo}, lH, mLv, lS, mSLv);
  mpsxx::compute_merged_operator(0, std::vector<QA4>{rmpo}, rH, mRv, rS, mSRv);
  const QA3& mL = mLv[0][0];
  const QA3& mR = mRv[0][0];
  write_qsd(dir + "/mL.ref.qsd", mL);
  write_qsd(dir + "/mR.ref.qsd", mR);

  // merged two-site wavefunction, the merge infos of src/optimize.hpp:548-557
  btas::QSTmergeInfo<2, fermion> q_lM, q_rM;
  {
    const btas::Qshapes<fermion>& q_l = -lopr.qshape(2);
    const btas::Qshapes<fermion>& q_m = -lmpo.qshape(2);
    q_lM.reset(btas::make_array(q_l, q_m), btas::make_array(lopr.dshape(0), lmpo.dshape(1)));
    const btas::Qshapes<fermion>& q_n = -rmpo.qshape(2);
    const btas::Qshapes<fermion>& q_r = -ropr.qshape(2);
    q_rM.reset(btas::make_array(q_n, q_r), btas::make_array(rmpo.dshape(1), ropr.dshape(0)));
  }
  QA4 twf;
  btas::Gemm(btas::NoTrans, btas::NoTrans, 1.0, lwfn, rwfn, 1.0, twf);
  QA2 psi;
  btas::QSTmerge(q_lM, twf, q_rM, psi);
  write_qsd(dir + "/psi.ref.qsd", psi);

  // sigma: the two Gemm's of compute_sigma_vector with the intermediate kept visible
  std::vector<std::vector<TaskRecord>> lists;
  mpsxx_ref::task_sink = &lists;
  QA3 scr1;
  btas::Gemm(btas::NoTrans, btas::NoTrans, 1.0, mL, psi, 1.0, scr1);
  QA2 sigma;
  btas::Gemm(btas::NoTrans, btas::Trans, 1.0, scr1, mR, 1.0, sigma);
  mpsxx_ref::task_sink = nullptr;
  QA2 sigma2;
  mpsxx::compute_sigma_vector(mL, mR, psi, sigma2);
  const double dsig = max_abs_diff(sigma, sigma2) + max_abs_diff(sigma2, sigma);
  write_qsd(dir + "/sigma.ref.qsd", sigma);
  {
    Registry rL, rPsi, rScr, rR, rSig;
    rL.add(mL), rPsi.add(psi), rScr.add(scr1), rR.add(mR), rSig.add(sigma);
    std::ofstream f(dir + "/tasks_sigma.ref.txt");
    write_tasks(f, "LxPsi", lists.at(0), rL, rPsi, rScr);
    write_tasks(f, "ScrxR", lists.at(1), rScr, rR, rSig);
  }

  // diagonal of H_eff over the blocks of psi
  QA2 diag(psi.q(), psi.qshape());
  mpsxx::compute_diagonal_elements(std::vector<QA3>{mL}, std::vector<QA3>{mR}, diag);
  write_qsd(dir + "/diag.ref.qsd", diag);

  // truncated SVD of psi
  QA2 wf(psi), lmat, rmat;
  mpsxx::canonicalize(forward, wf, lmat, rmat, M, 0.0);
  write_qsd(dir + "/lmat.ref.qsd", lmat);
  write_qsd(dir + "/rmat.ref.qsd", rmat);

  // renormalisation of the merged operator with the kept factor (bra = ket)
  lists.clear();
  const QA2& u = forward ? lmat : rmat;
  const QA3& mop = forward ? mL : mR;
  QA3 rscr, env;
  QA2 bra = u.conjugate();
  mpsxx_ref::task_sink = &lists;
  if (forward) {
    btas::Gemm(btas::Trans, btas::NoTrans, 1.0, bra, mop, 1.0, rscr);
    btas::Gemm(btas::NoTrans, btas::NoTrans, 1.0, rscr, u, 1.0, env);
  } else {
    btas::Gemm(btas::NoTrans, btas::NoTrans, 1.0, bra, mop, 1.0, rscr);
    btas::Gemm(btas::NoTrans, btas::Trans, 1.0, rscr, u, 1.0, env);
  }
  mpsxx_ref::task_sink = nullptr;
  QA3 env2;
  mpsxx::renormalize(forward, mop, u, u, env2);
  const double denv = max_abs_diff(env, env2) + max_abs_diff(env2, env);
  write_qsd(dir + "/env.ref.qsd", env);
  {
    Registry rBra, rOp, rScr, rU, rEnv;
    rBra.add(bra), rOp.add(mop), rScr.add(rscr), rU.add(u), rEnv.add(env);
    std::ofstream f(dir + "/tasks_renorm.ref.txt");
    write_tasks(f, "BraxOp", lists.at(0), rBra, rOp, rScr);
    write_tasks(f, "ScrxKet", lists.at(1), rScr, rU, rEnv);
  }
  std::printf("{\"dir\": \"%s\", \"sigma_check\": %.3e, \"renorm_check\": %.3e}\n", dir.c_str(), dsig, denv);
  return (dsig == 0.0 && denv == 0.0) ? 0 : 3;
}

int run_time_sigma(const std::string& dir, int steps) {
  QA3 mL, mR;
  QA2 psi;
  read_qsd(dir + "/mL.qsd", mL);
  read_qsd(dir + "/mR.qsd", mR);
  read_qsd(dir + "/psi.qsd", psi);
  std::vector<std::vector<TaskRecord>> lists;
  mpsxx_ref::task_sink = &lists;
  QA2 warm;
  mpsxx::compute_sigma_vector(mL, mR, psi, warm);
  mpsxx_ref::task_sink = nullptr;
  double flops = 0.0;
  for (const auto& l : lists)
    for (const auto& t : l) flops += t.flops;
  std::vector<double> dt;
  for (int s = 0; s < steps; ++s) {
    QA2 sigma;
    const auto t0 = std::chrono::steady_clock::now();
    mpsxx::compute_sigma_vector(mL, mR, psi, sigma);
    dt.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
  }
  double tot = 0.0;
  for (double x : dt) tot += x;
  std::printf("{\"steps\": %d, \"seconds_per_step\": %.6f, \"flops_per_step\": %.6e, \"threads\": %d}\n", steps,
              tot / std::max(1, steps), flops, omp_get_max_threads());
  return 0;
}

int run_dump_mpo(const std::string& prefix, int nsites, const std::string& outdir) {
  for (int i = 0; i < nsites; ++i) {
    std::vector<QA4> mpo;
    load(mpo, mpsxx::getfile("mpo", prefix, i));
    if (mpo.size() != 1) throw std::runtime_error("dump_mpo: expected one operator group");
    write_qsd(outdir + "/mpo_" + std::to_string(i) + ".qsd", mpo[0]);
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_ops.x ops <bond_dir> | time_sigma <dir> <steps>\n");
    return 2;
  }
  const std::string cmd = argv[1];
  try {
    if (cmd == "ops") return run_ops(argv[2]);
    if (cmd == "time_sigma") return run_time_sigma(argv[2], argc > 3 ? std::atoi(argv[3]) : 3);
    if (cmd == "dump_mpo" && argc > 4) return run_dump_mpo(argv[2], std::atoi(argv[3]), argv[4]);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_ops.x: %s\n", e.what());
    return 1;
  }
  std::fprintf(stderr, "ref_ops.x: unknown command %s\n", cmd.c_str());
  return 2;
}
