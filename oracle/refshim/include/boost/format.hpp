// Stand-in for boost::format as the reference uses it (log text only; TEST
// INFRASTRUCTURE ONLY): each % argument replaces the next printf-style directive,
// printed with the stream's default formatting.
#ifndef NOMAD_REFSHIM_BOOST_FORMAT_H_
#define NOMAD_REFSHIM_BOOST_FORMAT_H_

#include <ostream>
#include <sstream>
#include <string>

namespace boost {

class format {
 public:
  explicit format(const std::string& f) : rest_(f) {}
  template <typename T>
  format& operator%(const T& v) {
    const std::size_t p = next_directive();
    if (p == std::string::npos) {
      done_ += rest_;
      rest_.clear();
      return *this;
    }
    std::size_t e = p + 1;
    while (e < rest_.size() && std::string("diufFeEgGxXoscpaAn%").find(rest_[e]) == std::string::npos) ++e;
    std::ostringstream os;
    os << v;
    done_ += rest_.substr(0, p) + os.str();
    rest_ = e < rest_.size() ? rest_.substr(e + 1) : std::string();
    return *this;
  }
  std::string str() const { return done_ + rest_; }

 private:
  std::size_t next_directive() const {
    std::size_t p = rest_.find('%');
    while (p != std::string::npos && p + 1 < rest_.size() && rest_[p + 1] == '%') p = rest_.find('%', p + 2);
    return p;
  }
  std::string done_, rest_;
};

inline std::ostream& operator<<(std::ostream& os, const format& f) { return os << f.str(); }

}  // namespace boost

#endif
