// Minimal glog stand-in for the reference harness (test infrastructure).
#ifndef SG_REF_GLOG_STUB_H_
#define SG_REF_GLOG_STUB_H_
#include <cstdlib>
#include <iostream>
#include <sstream>

namespace sg_glog {
extern int min_level;  // 0 INFO, 1 WARNING, 2 ERROR, 3 FATAL
class Line {
 public:
  Line(int level, const char* file, int line) : level_(level) {
    if (level_ >= min_level) os_ << "[" << "IWEF"[level < 4 ? level : 3] << " " << file << ":" << line << "] ";
  }
  ~Line() {
    if (level_ >= min_level) {
      os_ << "\n";
      std::cerr << os_.str();
    }
    if (level_ >= 3) std::abort();
  }
  std::ostream& stream() { return os_; }

 private:
  int level_;
  std::ostringstream os_;
};
struct Void {
  void operator&(std::ostream&) {}
};
class Null {
 public:
  template <typename T>
  Null& operator<<(const T&) { return *this; }
  Null& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
}  // namespace sg_glog

#define SG_LOG_INFO 0
#define SG_LOG_WARNING 1
#define SG_LOG_ERROR 2
#define SG_LOG_FATAL 3
#define LOG(sev) ::sg_glog::Line(SG_LOG_##sev, __FILE__, __LINE__).stream()
#define VLOG(n) if (true) {} else ::sg_glog::Null()
#define DLOG(sev) if (true) {} else ::sg_glog::Null()
#define LOG_IF(sev, cond) if (!(cond)) {} else LOG(sev)
#define CHECK(cond) if (cond) {} else ::sg_glog::Line(3, __FILE__, __LINE__).stream() << "Check failed: " #cond " "
#define SG_CHECK_OP(a, b, op) CHECK((a) op (b))
#define CHECK_EQ(a, b) SG_CHECK_OP(a, b, ==)
#define CHECK_NE(a, b) SG_CHECK_OP(a, b, !=)
#define CHECK_LT(a, b) SG_CHECK_OP(a, b, <)
#define CHECK_LE(a, b) SG_CHECK_OP(a, b, <=)
#define CHECK_GT(a, b) SG_CHECK_OP(a, b, >)
#define CHECK_GE(a, b) SG_CHECK_OP(a, b, >=)
#define CHECK_NOTNULL(p) (p)

namespace google {
inline void InitGoogleLogging(const char*) {}
inline void ShutdownGoogleLogging() {}
inline void InstallFailureSignalHandler() {}
}  // namespace google
#endif
