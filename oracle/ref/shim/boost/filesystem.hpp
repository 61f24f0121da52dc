// boost::filesystem stand-in (path, exists, remove) over std::filesystem.
#ifndef MPSXX_REF_BOOST_FILESYSTEM_HPP
#define MPSXX_REF_BOOST_FILESYSTEM_HPP
#include <filesystem>
#include <boost/mpsxx_shim.hpp>
namespace boost {
namespace filesystem {
using std::filesystem::exists;
using std::filesystem::path;
using std::filesystem::remove;
}  // namespace filesystem
}  // namespace boost
#endif
