// No-op stand-in for <boost/log/trivial.hpp>, used ONLY to compile the reference's own
// source files (src/sim/kernels.cu, src/sim/config_reader.cpp) into the test oracle under
// oracle/_ref. Boost is not installed in this image. The reference uses exactly one macro,
// BOOST_LOG_TRIVIAL(severity) << ..., and relies on Boost pulling in a few std headers.
#pragma once
#include <cstring>
#include <iterator>
#include <sstream>
#include <ostream>

namespace sw_oracle_stub {
struct null_stream {
    template <typename T> null_stream &operator<<(const T &) { return *this; }
    null_stream &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
}  // namespace sw_oracle_stub

#define BOOST_LOG_TRIVIAL(severity) (sw_oracle_stub::null_stream{})
