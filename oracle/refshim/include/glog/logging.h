// Stand-in for glog's LOG(severity) stream macro (TEST INFRASTRUCTURE ONLY): INFO and
// WARNING are discarded, ERROR goes to stderr, FATAL aborts after printing.
#ifndef NOMAD_REFSHIM_GLOG_H_
#define NOMAD_REFSHIM_GLOG_H_

#include <cstdlib>
#include <iostream>
#include <sstream>

namespace refshim {
enum Severity { INFO = 0, WARNING = 1, ERROR = 2, FATAL = 3 };
class LogLine {
 public:
  explicit LogLine(int sev) : sev_(sev) {}
  ~LogLine() {
    if (sev_ >= ERROR) std::cerr << "[reference " << (sev_ == FATAL ? "FATAL" : "ERROR") << "] " << os_.str() << "\n";
    if (sev_ == FATAL) std::abort();
  }
  template <typename T>
  LogLine& operator<<(const T& v) {
    if (sev_ >= ERROR) os_ << v;
    return *this;
  }
  LogLine& operator<<(std::ostream& (*f)(std::ostream&)) {
    if (sev_ >= ERROR) os_ << f;
    return *this;
  }

 private:
  int sev_;
  std::ostringstream os_;
};
}  // namespace refshim

#define LOG(sev) ::refshim::LogLine(::refshim::sev)

namespace google {
inline void InitGoogleLogging(const char*) {}
}  // namespace google

#endif
