// Stand-ins for the few Boost facilities the mpsxx reference sources use, so that the
// reference builds here against the standard library alone.  Test infrastructure for
// the oracle: nothing in the product links it.
//
//  * smart pointers / function / bind       -> std:: equivalents;
//  * serialization + binary archives        -> a plain length-prefixed binary format,
//    enough to save and reload the reference's own disk state (src/fileio.h:9-25);
//  * MPI                                    -> one rank (broadcast is a no-op);
//  * filesystem / algorithm::string         -> std::filesystem and small helpers.
#ifndef MPSXX_REF_BOOST_SHIM_HPP
#define MPSXX_REF_BOOST_SHIM_HPP

#ifndef BOOST_VERSION
#define BOOST_VERSION 107000
#endif

#include <array>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace boost {
using std::shared_ptr;
using std::weak_ptr;
using std::function;
using std::bind;
template <class T, std::size_t N> using array = std::array<T, N>;

namespace serialization {

// Member serialize() is private and befriends this class; detection and calls go through it.
class access {
 public:
  template <class A, class T>
  static auto has_member(int) -> decltype(std::declval<T&>().serialize(std::declval<A&>(), 0u), std::true_type());
  template <class A, class T>
  static std::false_type has_member(...);
  template <class A, class T>
  static void call(A& ar, T& t) { t.serialize(ar, 0u); }
};

template <class Base, class Derived>
Base& base_object(Derived& d) { return static_cast<Base&>(d); }
template <class Base, class Derived>
const Base& base_object(const Derived& d) { return static_cast<const Base&>(d); }

}  // namespace serialization

namespace archive {
namespace detail {

// Writer and reader share one traversal; `io` moves raw bytes in either direction.
template <class Ar, class T>
typename std::enable_if<std::is_arithmetic<T>::value || std::is_enum<T>::value>::type walk(Ar& ar, T& t) {
  ar.io(&t, sizeof(T));
}
template <class Ar, class T>
void walk(Ar& ar, std::complex<T>& t) { ar.io(&t, sizeof(t)); }
template <class Ar>
void walk(Ar& ar, std::string& s) {
  std::uint64_t n = s.size();
  ar.io(&n, sizeof(n));
  if (Ar::is_loading) s.resize(n);
  if (n) ar.io(&s[0], n);
}
template <class Ar, class T, class A>
void walk(Ar& ar, std::vector<T, A>& v);
template <class Ar, class K, class V, class C, class A>
void walk(Ar& ar, std::map<K, V, C, A>& m);
template <class Ar, class T, std::size_t N>
void walk(Ar& ar, std::array<T, N>& a);
template <class Ar, class T>
void walk(Ar& ar, std::shared_ptr<T>& p);
template <class Ar, class A, class B>
void walk(Ar& ar, std::pair<A, B>& p);
template <class Ar, class T>
typename std::enable_if<decltype(serialization::access::has_member<Ar, T>(0))::value>::type walk(Ar& ar, T& t) {
  serialization::access::call(ar, t);
}

template <class Ar, class T, class A>
void walk(Ar& ar, std::vector<T, A>& v) {
  std::uint64_t n = v.size();
  ar.io(&n, sizeof(n));
  if (Ar::is_loading) v.resize(n);
  for (auto& x : v) walk(ar, x);
}
template <class Ar, class K, class V, class C, class A>
void walk(Ar& ar, std::map<K, V, C, A>& m) {
  std::uint64_t n = m.size();
  ar.io(&n, sizeof(n));
  if (Ar::is_loading) {
    m.clear();
    for (std::uint64_t i = 0; i < n; ++i) {
      K k{};
      V v{};
      walk(ar, k);
      walk(ar, v);
      m.emplace_hint(m.end(), std::move(k), std::move(v));
    }
  } else {
    for (auto& kv : m) {
      K k = kv.first;
      walk(ar, k);
      walk(ar, kv.second);
    }
  }
}
template <class Ar, class T, std::size_t N>
void walk(Ar& ar, std::array<T, N>& a) {
  for (auto& x : a) walk(ar, x);
}
template <class Ar, class T>
void walk(Ar& ar, std::shared_ptr<T>& p) {
  unsigned char has = p ? 1 : 0;
  ar.io(&has, 1);
  if (Ar::is_loading) p = has ? std::make_shared<T>() : std::shared_ptr<T>();
  if (has) walk(ar, *p);
}
template <class Ar, class A, class B>
void walk(Ar& ar, std::pair<A, B>& p) {
  walk(ar, p.first);
  walk(ar, p.second);
}

}  // namespace detail

class binary_oarchive {
 public:
  static const bool is_loading = false;
  static const bool is_saving = true;
  explicit binary_oarchive(std::ostream& os) : os_(os) {}
  void io(const void* p, std::size_t n) {
    os_.write(static_cast<const char*>(p), static_cast<std::streamsize>(n));
    if (!os_) throw std::runtime_error("binary_oarchive: write failed");
  }
  template <class T>
  binary_oarchive& operator&(const T& t) {
    detail::walk(*this, const_cast<T&>(t));
    return *this;
  }
  template <class T>
  binary_oarchive& operator<<(const T& t) { return *this & t; }

 private:
  std::ostream& os_;
};

class binary_iarchive {
 public:
  static const bool is_loading = true;
  static const bool is_saving = false;
  explicit binary_iarchive(std::istream& is) : is_(is) {}
  void io(void* p, std::size_t n) {
    is_.read(static_cast<char*>(p), static_cast<std::streamsize>(n));
    if (!is_) throw std::runtime_error("binary_iarchive: read failed (missing or short file)");
  }
  template <class T>
  binary_iarchive& operator&(T& t) {
    detail::walk(*this, t);
    return *this;
  }
  template <class T>
  binary_iarchive& operator>>(T& t) { return *this & t; }

 private:
  std::istream& is_;
};

}  // namespace archive

namespace mpi {
// One rank: every collective is the identity; point-to-point calls never happen
// (the reference only sends from ranks other than 0).
struct environment {
  environment() {}
  environment(int, char**) {}
};
struct communicator {
  int rank() const { return 0; }
  int size() const { return 1; }
  template <class T>
  void send(int, int, const T&) const { throw std::logic_error("mpi shim: send on a single rank"); }
  template <class T>
  void recv(int, int, T&) const { throw std::logic_error("mpi shim: recv on a single rank"); }
};
template <class T>
void broadcast(const communicator&, T&, int) {}
template <class T, class Op>
void all_reduce(const communicator&, const T& in, T& out, Op) { out = in; }
}  // namespace mpi

}  // namespace boost

using std::placeholders::_1;
using std::placeholders::_2;
using std::placeholders::_3;
using std::placeholders::_4;

#endif
