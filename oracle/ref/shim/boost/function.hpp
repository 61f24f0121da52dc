#include <boost/mpsxx_shim.hpp>
