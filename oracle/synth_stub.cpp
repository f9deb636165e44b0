// TEST INFRASTRUCTURE ONLY: lets the library's synthetic phantom generator
// (spinwalk_gb300/csrc/sw_phantom.cpp) link on its own into oracle/libsynth.so. In the library,
// sw::api::fail also records the message for sw_last_error(); here the message goes to stderr.
#include <cstdio>
#include <string>

namespace sw {
namespace api {
int fail(int code, const std::string &msg) {
    std::fprintf(stderr, "libsynth: %s\n", msg.c_str());
    return code;
}
}  // namespace api
}  // namespace sw
