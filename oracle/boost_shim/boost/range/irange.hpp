// Stand-in for boost::irange, the only Boost facility the reference's Utils.hpp uses: an
// integer half-open range [first, last) for range-based for loops. Written for this project
// (test infrastructure only); it lets oracle/ref_build.sh compile the reference's
// BoundingBox, Nint and LinkListOrtho from the reference tree without Boost.
#pragma once

namespace boost {

template <class T>
class shim_integer_range {
 public:
  class iterator {
   public:
    explicit iterator(T v) : v_(v) {}
    T operator*() const { return v_; }
    iterator &operator++() {
      ++v_;
      return *this;
    }
    bool operator!=(const iterator &o) const { return v_ != o.v_; }

   private:
    T v_;
  };
  shim_integer_range(T first, T last) : first_(first), last_(last < first ? first : last) {}
  iterator begin() const { return iterator(first_); }
  iterator end() const { return iterator(last_); }

 private:
  T first_, last_;
};

template <class T, class U>
shim_integer_range<T> irange(T first, U last) {
  return shim_integer_range<T>(first, static_cast<T>(last));
}

}  // namespace boost
