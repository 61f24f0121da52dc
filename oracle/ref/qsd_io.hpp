// Block-sparse tensor files shared by the reference harness (C++) and the oracle
// (oracle/ref_io.py).  Little-endian:
//   "MQSD" | int32 rank | int32 q.p, q.s | per index: int32 nsec, nsec x (int32 p, s, dim)
//   | int64 nblocks | per block: int64 tag, int64 size, size x float64 (row-major)
// Oracle test infrastructure.
#ifndef MPSXX_REF_QSD_IO_HPP
#define MPSXX_REF_QSD_IO_HPP

#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>

#include <btas/QSPARSE/QSTArray.h>

#include "fermion.h"

namespace mpsxx_ref {

template <size_t N>
void write_qsd(const std::string& path, const btas::QSTArray<double, N, fermion>& a) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("write_qsd: cannot open " + path);
  auto put32 = [&](int32_t v) { f.write(reinterpret_cast<const char*>(&v), 4); };
  auto put64 = [&](int64_t v) { f.write(reinterpret_cast<const char*>(&v), 8); };
  f.write("MQSD", 4);
  put32(static_cast<int32_t>(N));
  put32(a.q().p());
  put32(a.q().s());
  for (size_t i = 0; i < N; ++i) {
    const auto& qs = a.qshape(i);
    const auto& ds = a.dshape(i);
    put32(static_cast<int32_t>(qs.size()));
    for (size_t k = 0; k < qs.size(); ++k) {
      put32(qs[k].p());
      put32(qs[k].s());
      put32(k < ds.size() ? ds[k] : 0);
    }
  }
  int64_t nb = 0;
  for (auto it = a.begin(); it != a.end(); ++it)
    if (it->second) ++nb;
  put64(nb);
  for (auto it = a.begin(); it != a.end(); ++it) {
    if (!it->second) continue;
    put64(it->first);
    put64(static_cast<int64_t>(it->second->size()));
    f.write(reinterpret_cast<const char*>(it->second->data()), sizeof(double) * it->second->size());
  }
  if (!f) throw std::runtime_error("write_qsd: write failed for " + path);
}

template <size_t N>
void read_qsd(const std::string& path, btas::QSTArray<double, N, fermion>& a) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("read_qsd: cannot open " + path);
  auto get32 = [&]() { int32_t v; f.read(reinterpret_cast<char*>(&v), 4); return v; };
  auto get64 = [&]() { int64_t v; f.read(reinterpret_cast<char*>(&v), 8); return v; };
  char magic[4];
  f.read(magic, 4);
  if (std::memcmp(magic, "MQSD", 4) != 0) throw std::runtime_error("read_qsd: bad magic in " + path);
  if (get32() != static_cast<int32_t>(N)) throw std::runtime_error("read_qsd: rank mismatch in " + path);
  const int qp = get32(), qs_ = get32();
  btas::TVector<btas::Qshapes<fermion>, N> qshape;
  btas::TVector<btas::Dshapes, N> dshape;
  for (size_t i = 0; i < N; ++i) {
    const int ns = get32();
    for (int k = 0; k < ns; ++k) {
      const int p = get32(), s = get32(), d = get32();
      qshape[i].push_back(fermion(p, s));
      dshape[i].push_back(d);
    }
  }
  a.resize(fermion(qp, qs_), qshape, dshape, false);
  const int64_t nb = get64();
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t tag = get64(), size = get64();
    auto it = a.reserve(static_cast<int>(tag));
    if (static_cast<int64_t>(it->second->size()) != size)
      throw std::runtime_error("read_qsd: block size mismatch in " + path);
    f.read(reinterpret_cast<char*>(it->second->data()), sizeof(double) * size);
  }
  if (!f) throw std::runtime_error("read_qsd: short file " + path);
}

}  // namespace mpsxx_ref

#endif
