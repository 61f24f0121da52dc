// Definitions behind hooks.hpp: the task-list sink and the bond-dumping overload of
// optimize_twosite_merged.  Oracle test infrastructure.
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <string>

#include "hooks.hpp"
#include "qsd_io.hpp"

namespace mpsxx_ref {
std::vector<std::vector<TaskRecord>>* task_sink = nullptr;
}

namespace mpsxx {

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
                               const int& M, const double& noise) {
  static long seq = 0;
  const char* root = std::getenv("MPSXX_REF_DUMP");
  const size_t r = lWfnc.size() - 1;
  std::string dir;
  if (root) {
    char name[32];
    std::snprintf(name, sizeof(name), "bond_%05ld", seq);
    dir = std::string(root) + "/" + name;
    std::filesystem::create_directories(dir);
    using mpsxx_ref::write_qsd;
    write_qsd(dir + "/lmpo.qsd", lmpo[0]);
    write_qsd(dir + "/rmpo.qsd", rmpo[0]);
    write_qsd(dir + "/lopr.qsd", lHopr[r][0]);
    write_qsd(dir + "/ropr.qsd", rHopr[r][0]);
    write_qsd(dir + "/lsopr.qsd", lSopr[r]);
    write_qsd(dir + "/rsopr.qsd", rSopr[r]);
    write_qsd(dir + "/lwfn.qsd", lWfnc[r]);
    write_qsd(dir + "/rwfn.qsd", rWfnc[r]);
  }
  const double e = optimize_twosite_merged<fermion>(forward, E, lmpo, rmpo, lHopr, rHopr, lSopr, rSopr, kMps, lWfnc,
                                                    rWfnc, tole, M, noise);
  if (root) {
    using mpsxx_ref::write_qsd;
    write_qsd(dir + "/out_env.qsd", forward ? lHopr[r][0] : rHopr[r][0]);
    write_qsd(dir + "/out_senv.qsd", forward ? lSopr[r] : rSopr[r]);
    write_qsd(dir + "/out_lwfn.qsd", lWfnc[r]);
    write_qsd(dir + "/out_rwfn.qsd", rWfnc[r]);
    std::ofstream meta(dir + "/meta.txt");
    meta << std::setprecision(17) << "forward " << int(forward) << "\nM " << M << "\ntole " << tole << "\nnoise "
         << noise << "\nngroups " << lmpo.size() << "\nroots " << lWfnc.size() << "\nenergy " << e << "\n";
  }
  ++seq;
  return e;
}

}  // namespace mpsxx
