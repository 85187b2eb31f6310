// Stand-in for boost::format, which the reference's Utils.hpp includes and its Common.hpp
// names (printArray). Test infrastructure only: the reference code compiled here (box,
// link list, force laws) never formats, so a class that accepts arguments through % and
// prints them one after another is enough to compile it without Boost.
#pragma once
#include <ostream>
#include <sstream>
#include <string>

namespace boost {

class format {
 public:
  explicit format(const char *) {}
  explicit format(const std::string &) {}
  template <class T>
  format &operator%(const T &v) {
    std::ostringstream o;
    o << v;
    text_ += o.str();
    return *this;
  }
  std::string str() const { return text_; }

 private:
  std::string text_;
};

inline std::ostream &operator<<(std::ostream &o, const format &f) { return o << f.str(); }

}  // namespace boost
