// Definitions behind the glog / gflags stand-ins and no-op definitions of
// the reference's CUDA shim entry points (the harness runs the CPU path with
// -gpu_start=0; none of these is needed for its results).
#include <glog/logging.h>
#include <gflags/gflags.h>

namespace sg_glog {
int min_level = 0;
}
namespace sg_gflags {
std::map<std::string, std::function<void(const std::string&)>>& registry() {
  static std::map<std::string, std::function<void(const std::string&)>> r;
  return r;
}
bool Set(const std::string& name, const std::string& value) {
  auto it = registry().find(name);
  if (it == registry().end()) return false;
  it->second(value);
  return true;
}
}  // namespace sg_gflags
