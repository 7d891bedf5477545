// Minimal gflags stand-in: DEFINE_* create globals registered for
// sg_gflags::Set(name, value) (used by the harness driver to set flags).
#ifndef SG_REF_GFLAGS_STUB_H_
#define SG_REF_GFLAGS_STUB_H_
#include <cstdint>
#include <cstdlib>
#include <functional>
#include <map>
#include <string>

#include "gflags_declare.h"

namespace sg_gflags {
std::map<std::string, std::function<void(const std::string&)>>& registry();
struct Reg {
  Reg(const char* name, std::function<void(const std::string&)> f) { registry()[name] = f; }
};
bool Set(const std::string& name, const std::string& value);
}  // namespace sg_gflags

#define SG_GFLAG_DEFINE(type, n, def, conv)                                            \
  type FLAGS_##n = def;                                                                 \
  static ::sg_gflags::Reg sg_reg_##n(#n, [](const std::string& v) { FLAGS_##n = conv; })
#define DEFINE_bool(n, def, desc) SG_GFLAG_DEFINE(bool, n, def, (v == "true" || v == "1"))
#define DEFINE_int32(n, def, desc) SG_GFLAG_DEFINE(int32_t, n, def, (int32_t)std::stol(v))
#define DEFINE_int64(n, def, desc) SG_GFLAG_DEFINE(int64_t, n, def, (int64_t)std::stoll(v))
#define DEFINE_uint64(n, def, desc) SG_GFLAG_DEFINE(uint64_t, n, def, (uint64_t)std::stoull(v))
#define DEFINE_double(n, def, desc) SG_GFLAG_DEFINE(double, n, def, std::stod(v))
#define DEFINE_string(n, def, desc) SG_GFLAG_DEFINE(std::string, n, def, v)

namespace google {
inline void SetUsageMessage(const std::string&) {}
inline void ShowUsageWithFlagsRestrict(const char*, const char*) {}
inline void ParseCommandLineFlags(int*, char***, bool) {}
inline void ShutDownCommandLineFlags() {}
}  // namespace google
#endif
